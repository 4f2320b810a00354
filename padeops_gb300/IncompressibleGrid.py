"""Mirror of module IncompressibleGrid (src/incompressible/igrid.F90): type igrid, restricted
to the periodic-in-z LES configuration this library provides.

Fourier x/y, staggered CD06 z, rotational advection, TVD-RK3, viscosity 1/Re, and the
Smagorinsky model with the standard dynamic procedure.  Parameters that the reference
reads from its namelist input file are keyword arguments here; fields are CUDA torch
tensors in Fortran order (x fastest): u, v (nx, ny, nz), w on the nz+1 edges.
"""
import ctypes

import numpy as np

from . import _lib as L
from .spectralMod import _dev

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def restart_name(rid, var, tid):
    """RESTART file name (igrid.F90:2729, 2775): format (A7,A4,I2.2,A3,I6.6), and
    (A7,A4,I2.2,A6,I6.6) for the info file."""
    return f"RESTART_Run{rid:02d}_{var}.{tid:06d}"


def fortran_g15_5(x):
    """Fortran list item of format (100g15.5) for one real (the restart info file): F editing
    with 5 significant digits and 4 trailing blanks when 0.1 <= |x| < 1e5 after rounding,
    E15.5 otherwise."""
    x = float(x)
    if x == 0.0:
        return f"{'0.0000':>11}    "
    r = float(f"{abs(x):.5g}") if np.isfinite(x) else abs(x)
    if np.isfinite(x) and 0.1 <= r < 1e5:
        k = int(np.floor(np.log10(r))) + 1  # digits before the decimal point
        if k == 5:  # F11.0 keeps the decimal point
            return f"{f'{x:.0f}.':>11}    "
        return f"{x:11.{5 - k}f}    "
    m, e = f"{abs(x):.4e}".split("e")  # d.dddd e+XX -> 0.ddddd E+(XX+1)
    mant = "0." + m.replace(".", "")
    ex = int(e) + 1
    return f"{('-' if x < 0 else '') + mant + ('E+' if ex >= 0 else 'E-') + f'{abs(ex):02d}':>15}"


class igrid:
    def __init__(self):
        self._h = ctypes.c_void_p(None)

    def init(self, nx, ny, nz, Lx=2 * np.pi, Ly=2 * np.pi, Lz=2 * np.pi, Re=1000.0, isInviscid=False, CFL=0.5,
             dt=-1.0, useSGS=True, DynamicProcedureType=1, Csgs=0.17, deltaRatio=2.0, DynProcFreq=1,
             dealiasFact=2.0 / 3.0, t_DivergenceCheck=10, learnedSGS=False, JudgeFreq=0, learnedPlaneAvg=False,
             SGSModelID=0, JudgeTol=0.0):
        """igrid init (igrid.F90:330-660) for PeriodicInZ with SGSModelID 0 (Smagorinsky).

        learnedSGS replaces the model coefficient by the learned closure (set_mlp), with the
        dynamic procedure run every JudgeFreq steps as its judge (0: never): judge_info gives
        the closure's error against it, its lambda(z) is the fallback coefficient of points
        outside the closure's training range, and while the error exceeds JudgeTol (> 0)
        every point takes that fallback;
        learnedPlaneAvg applies the closure's coefficient averaged over each x-y plane, the
        form of the dynamic procedure's lambda(z), instead of pointwise.  SGSModelID: 0
        Smagorinsky, 1 sigma, 2 AMD (the last two with DynamicProcedureType 0)."""
        if DynamicProcedureType not in (0, 1):
            raise L.PadeError(L.PADE_ENOTSUP, "only DynamicProcedureType 0 or 1")
        self.destroy()
        p = L.LesParams(nx, ny, nz, Lx, Ly, Lz, Re, int(bool(isInviscid)), CFL, dt, int(bool(useSGS)),
                        int(DynamicProcedureType == 1), Csgs, deltaRatio, DynProcFreq, dealiasFact,
                        t_DivergenceCheck, int(bool(learnedSGS)), int(JudgeFreq), int(bool(learnedPlaneAvg)),
                        int(SGSModelID), float(JudgeTol))
        self.Lx, self.Ly, self.Lz, self.Re = Lx, Ly, Lz, Re
        h = ctypes.c_void_p(None)
        L.check(L.lib().pade_les_init(ctypes.byref(h), ctypes.byref(p)), "igrid.init")
        self._h = h
        self.nx, self.ny, self.nz = nx, ny, nz

    @property
    def handle(self):
        if not self._h.value:
            raise L.PadeError(L.PADE_EINVAL, "igrid used before init")
        return self._h

    def set_fields(self, u, v, w):
        pu, _, s = _dev(u, "u")
        pv, _, _ = _dev(v, "v")
        pw, _, _ = _dev(w, "w")
        L.check(L.lib().pade_les_set_fields(self.handle, pu, pv, pw, s), "igrid.set_fields")

    def set_mlp(self, closure):
        """Attach a sgs_learned.LearnedClosure (kept alive by this object)."""
        self._closure = closure
        L.check(L.lib().pade_les_set_mlp(self.handle, closure.handle), "igrid.set_mlp")

    def timeAdvance(self, use_graph=True):
        """One TVD_RK3 step (TimeSteppingScheme 1) on torch's current stream."""
        s = torch.cuda.current_stream().cuda_stream if torch is not None else None
        L.check(L.lib().pade_les_step(self.handle, int(bool(use_graph)), s), "igrid.timeAdvance")

    def info(self):
        dt, ts, st = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        lam = np.empty(self.nz)
        L.check(L.lib().pade_les_info(self.handle, ctypes.byref(dt), ctypes.byref(ts), ctypes.byref(st),
                                      lam.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return {"dt": dt.value, "tsim": ts.value, "step": st.value, "lambda": lam}

    def judge_info(self):
        """The learned closure's judge: relative error of the last judge step (-1 before
        any), the closure's plane-averaged Cs^2 Delta^2 there, and the number of point
        evaluations that took the fallback coefficient."""
        err = ctypes.c_double()
        lam = np.empty(self.nz)
        nfb = ctypes.c_longlong()
        L.check(L.lib().pade_les_judge_info(self.handle, ctypes.byref(err),
                                            lam.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(nfb)),
                "igrid.judge_info")
        return {"err": err.value, "lambda_closure": lam, "n_fallback": nfb.value}

    def field(self, name):
        """A copy of an internal field as a CUDA tensor (Fortran-shaped view reversed)."""
        nx, ny, nz = self.nx, self.ny, self.nz
        nxh = nx // 2 + 1
        shapes = {"uhat": ((nz, ny, nxh), True), "vhat": ((nz, ny, nxh), True), "what": ((nz + 1, ny, nxh), True),
                  "u": ((nz, ny, nx), False), "v": ((nz, ny, nx), False), "wC": ((nz, ny, nx), False),
                  "w": ((nz + 1, ny, nx), False), "uE": ((nz + 1, ny, nx), False), "vE": ((nz + 1, ny, nx), False),
                  "nu_sgs_C": ((nz, ny, nx), False), "nu_sgs_E": ((nz + 1, ny, nx), False)}
        if name.startswith("duidxjC") or name.startswith("duidxjE"):
            idx = int(name[7:]) - 1
            which = (10 if name[6] == "C" else 20) + idx
            shape, cplx = ((nz if name[6] == "C" else nz + 1, ny, nx), False)
        else:
            which = L.LES_FIELDS[name]
            shape, cplx = shapes[name]
        p = ctypes.c_void_p(None)
        L.check(L.lib().pade_les_field(self.handle, which, ctypes.byref(p)))
        n = int(np.prod(shape)) * (2 if cplx else 1)
        t = torch.empty(n, dtype=torch.float64, device="cuda")
        # one-rank transpose = device copy of n doubles, ordered on the current stream
        L.check(L.lib().pade_transpose(1, 2, p, ctypes.c_void_p(t.data_ptr()), n, 1, 1, 8,
                                       torch.cuda.current_stream().cuda_stream))
        return (t.view(torch.complex128) if cplx else t).view(shape)

    def scalar_sgs(self, T, That, dTdxC, dTdyC, dTdzC, dTdzE, Trhs, Pr=1.0, dynamic=False):
        """getRHS_SGS_Scalar (sgsmod_igrid.F90:268-335) for a scalar carried beside the LES:
        Trhs (its x-y spectrum at the cells, complex) loses the divergence of the SGS flux
        -kappa grad T; kappa = nu_sgs / Pr, or Beta(z) |S| from the scalar dynamic procedure
        (standardDynamicProcedure.F90:1-71).  CUDA tensors in the layout of field(); returns
        Beta(z) (numpy) when dynamic."""
        beta = np.zeros(self.nz) if dynamic else None

        def vp(t):
            return ctypes.c_void_p(t.data_ptr())

        bp = beta.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if dynamic else None
        L.check(L.lib().pade_les_scalar_sgs(self.handle, vp(T), vp(That), vp(dTdxC), vp(dTdyC), vp(dTdzC),
                                            vp(dTdzE), vp(Trhs), float(Pr), int(bool(dynamic)),
                                            ctypes.cast(bp, ctypes.c_void_p) if dynamic else None,
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                "igrid.scalar_sgs")
        return beta

    def set_time(self, tsim, step):
        L.check(L.lib().pade_les_set_time(self.handle, float(tsim), int(step)), "igrid.set_time")

    def dumpRestartFile(self, OutputDir, runID=0):
        """igrid.F90:2767-2802: u, v (nx, ny, nz) and w (nx, ny, nz+1) as raw FP64 in the
        global x-pencil order of decomp_2d_write_one (column-major, x fastest), and tsim in
        the _info file; named by runID and the current step.  Returns the step."""
        import os

        inf = self.info()
        step = inf["step"]
        for var in ("u", "v", "w"):
            self.field(var).cpu().numpy().tofile(os.path.join(OutputDir, restart_name(runID, var, step)))
        with open(os.path.join(OutputDir, restart_name(runID, "info", step)), "w") as fh:
            fh.write(fortran_g15_5(inf["tsim"]) + "\n")
        return step

    def readRestartFile(self, InputDir, tid, rid):
        """igrid.F90:2719-2765 (u, v, w and tsim), with the step continuing from tid as
        the reference's init does after reading a restart.  The fields pass through
        set_fields (transform, dealias, projection: a no-op for a projected field)."""
        import os

        nx, ny, nz = self.nx, self.ny, self.nz
        arrs = {}
        for var, nzz in (("u", nz), ("v", nz), ("w", nz + 1)):
            a = np.fromfile(os.path.join(InputDir, restart_name(rid, var, tid)), dtype=np.float64)
            if a.size != nx * ny * nzz:
                raise L.PadeError(L.PADE_EINVAL, f"readRestartFile: {var} has {a.size} values, expected "
                                                 f"{nx * ny * nzz}")
            arrs[var] = torch.from_numpy(a.reshape(nzz, ny, nx)).cuda()
        with open(os.path.join(InputDir, restart_name(rid, "info", tid))) as fh:
            tsim = float(fh.readline()[:15].replace("D", "E").replace("d", "e"))
        self.set_fields(arrs["u"], arrs["v"], arrs["w"])
        self.set_time(tsim, tid)
        return tsim

    def destroy(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().pade_les_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
