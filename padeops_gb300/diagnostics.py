"""Flow statistics of an igrid LES, computed on the device from the solver's own fields.

* energy_spectrum: the 3-D kinetic-energy spectrum on integer wavenumber shells
  |k| in [s - 1/2, s + 1/2), from the solver's x-y Fourier coefficients (uhat, vhat, what)
  transformed along z with the library's FFT (pade_fft_c2c); normalised so that its sum is
  the kinetic energy 1/2 <u_i u_i> of the physical fields (Parseval).
* dissipation: the resolved viscous rate 2 nu <S_ij S_ij> and the SGS rate
  <2 nu_sgs S_ij S_ij> at the cell centres, from the solver's velocity gradients of its last
  stage (duidxjC1..9 = du/dx, du/dy, du/dz, dv/dx, ..., dw/dz).
* compare_spectra: per-shell relative deviation of one spectrum from another over the
  shells a run resolves (1 .. the 2/3 dealiasing cutoff).

The domain is 2 pi periodic in every direction (integer wavenumbers), as in the igrid
periodic configuration.
"""
import ctypes

import numpy as np

from . import _lib as L

try:
    import torch
except ImportError:  # pragma: no cover - CPU-only environments without torch
    torch = None


def _stream():
    return torch.cuda.current_stream().cuda_stream


def kinetic_energy(g):
    """1/2 <u^2 + v^2 + w^2> over the cells (w interpolated to the centres by the solver)."""
    s = 0.0
    for name in ("u", "v", "wC"):
        f = g.field(name)
        s += float((f * f).mean())
    return 0.5 * s


def energy_spectrum(g):
    """E(s) for shells s = 0 .. max, numpy array; sum(E) equals kinetic_energy(g)."""
    nx, ny, nz = g.nx, g.ny, g.nz
    nxh = nx // 2 + 1
    power = None
    lib = L.lib()
    for name in ("uhat", "vhat", "what"):
        h = g.field(name)[:nz].contiguous()  # (nz, ny, nxh); what: the nz distinct edge planes
        hk = torch.empty_like(h)
        L.check(lib.pade_fft_c2c(3, -1, ctypes.c_void_p(h.data_ptr()), ctypes.c_void_p(hk.data_ptr()), nxh, ny, nz,
                                 1.0, _stream()), "energy_spectrum")
        p = hk.real ** 2 + hk.imag ** 2
        power = p if power is None else power + p
    dev = power.device
    wx = torch.full((nxh,), 2.0, dtype=torch.float64, device=dev)  # r2c half spectrum: +-kx
    wx[0] = 1.0
    if nx % 2 == 0:
        wx[-1] = 1.0
    kx = torch.arange(nxh, dtype=torch.float64, device=dev)
    ky = torch.fft.fftfreq(ny, d=1.0 / ny, dtype=torch.float64, device=dev)
    kz = torch.fft.fftfreq(nz, d=1.0 / nz, dtype=torch.float64, device=dev)
    kk = torch.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    shell = torch.round(kk).long().flatten()
    e = torch.bincount(shell, weights=(power * wx[None, None, :]).flatten())
    e = e.cpu().numpy()
    ke = kinetic_energy(g)
    return e * (ke / e.sum()) if e.sum() > 0 else e


def dissipation(g, nu):
    """(resolved 2 nu <S_ij S_ij>, SGS <2 nu_sgs S_ij S_ij>) at the cell centres."""
    grads = [g.field(f"duidxjC{k + 1}") for k in range(9)]
    ss = None
    for i in range(3):
        for j in range(3):
            sij = 0.5 * (grads[3 * i + j] + grads[3 * j + i])
            t = sij * sij
            ss = t if ss is None else ss + t
    nus = g.field("nu_sgs_C")
    return 2.0 * nu * float(ss.mean()), 2.0 * float((nus * ss).mean())


def compare_spectra(e, ref, n, floor=0.0):
    """Relative deviation |e / ref - 1| per shell over shells 1 .. floor(n / 3) (the 2/3
    dealiasing cutoff of an n^3 run), restricted to the shells whose reference energy is at
    least `floor` times the largest (a flow that has not yet filled its high shells holds
    round-off there): dict with the max, the mean, the last shell compared and the
    per-shell array (NaN outside the compared shells)."""
    kc = n // 3
    e = np.asarray(e[1:kc + 1], dtype=float)
    r0 = np.asarray(ref[1:kc + 1], dtype=float)
    ok = r0 >= floor * r0.max()
    r = np.full(kc, np.nan)
    r[ok] = np.abs(e[ok] / r0[ok] - 1.0)
    last = int(np.nonzero(ok)[0].max()) + 1 if ok.any() else 0
    return {"max": float(np.nanmax(r)), "mean": float(np.nanmean(r)), "kmax": last, "per_shell": r}
