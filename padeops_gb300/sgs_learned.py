"""Learned SGS closure (no counterpart in the reference): an MLP 10 -> 64 -> 64 -> 1 that
predicts the Smagorinsky coefficient Cs^2 from the local velocity gradients, trained on
the dynamic procedure's coefficient and used by the LES step in its place.

``LearnedClosure`` owns the device parameters (``pade_mlp``); ``training_set`` gathers
(features, target) pairs from an LES run with the dynamic procedure; ``train`` runs AdamW
on the GPU.  Arrays are CUDA torch tensors.
"""
import ctypes

import numpy as np

from . import _lib as L

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

NPARAM = L.MLP_NPARAM


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _grads(ptrs):
    arr = (ctypes.c_void_p * 9)(*[p if isinstance(p, int) else p.data_ptr() for p in ptrs])
    return ctypes.cast(arr, ctypes.POINTER(ctypes.c_void_p))


def init_params(seed):
    """Seeded initial parameters: weights uniform in +-1/sqrt(fan_in), biases 0, and b3 such
    that the initial output is Cs^2 = 0.02."""
    rng = np.random.default_rng(seed)
    parts = [rng.uniform(-1, 1, (64, 10)) / np.sqrt(10), np.zeros(64), rng.uniform(-1, 1, (64, 64)) / 8.0,
             np.zeros(64), rng.uniform(-1, 1, 64) / 8.0, np.array([np.log(np.expm1(0.02))])]
    return np.concatenate([a.ravel() for a in parts]).astype(np.float32)


def delta_les(dx, dy, dz):
    """Filter width of the periodic-z Smagorinsky model (smagorinsky.F90:13-16)."""
    return (1.5 * dx * 1.5 * dy * 1.5 * dz) ** (1.0 / 3.0)


class LearnedClosure:
    def __init__(self, params=None):
        h = ctypes.c_void_p(None)
        L.check(L.lib().pade_mlp_create(ctypes.byref(h)), "pade_mlp_create")
        self._h = h
        if params is not None:
            self.set_params(params)

    @property
    def handle(self):
        return self._h

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != NPARAM:
            raise ValueError(f"expected {NPARAM} parameters")
        L.check(L.lib().pade_mlp_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def get_params(self):
        p = np.empty(NPARAM, dtype=np.float32)
        L.check(L.lib().pade_mlp_get_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return p

    def set_range(self, lo, hi):
        """Training range of the 10 features (None, None: no range).  Inside the LES, points
        outside it take the fallback coefficient instead of the network's."""
        if lo is None and hi is None:
            L.check(L.lib().pade_mlp_set_range(self._h, None, None), "pade_mlp_set_range")
            return
        lo = np.ascontiguousarray(lo, dtype=np.float32)
        hi = np.ascontiguousarray(hi, dtype=np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        L.check(L.lib().pade_mlp_set_range(self._h, lo.ctypes.data_as(fp), hi.ctypes.data_as(fp)),
                "pade_mlp_set_range")

    def loss_grad(self, X, y):
        loss = ctypes.c_float()
        g = np.empty(NPARAM, dtype=np.float32)
        L.check(L.lib().pade_mlp_loss_grad(self._h, _vp(X), _vp(y), int(y.numel()), ctypes.byref(loss),
                                           g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), _stream()))
        return loss.value, g

    def train_step(self, X, y, lr=1e-3, wd=0.0, want_loss=False):
        loss = ctypes.c_float()
        L.check(L.lib().pade_mlp_train_step(self._h, _vp(X), _vp(y), int(y.numel()), lr, wd,
                                            ctypes.byref(loss) if want_loss else None, _stream()))
        return loss.value if want_loss else None

    def features(self, grads, delta, nu):
        n = grads[0].numel()
        X = torch.empty((n, 10), dtype=torch.float32, device=grads[0].device)
        L.check(L.lib().pade_mlp_features(_grads(grads), n, delta, nu, _vp(X), _stream()))
        return X

    def infer_nu(self, grads, delta, nu, want_cs2=False):
        n = grads[0].numel()
        out = torch.empty(n, dtype=torch.float64, device=grads[0].device)
        cs2 = torch.empty(n, dtype=torch.float32, device=grads[0].device) if want_cs2 else None
        L.check(L.lib().pade_mlp_infer_nu(self._h, _grads(grads), n, delta, nu, _vp(out),
                                          _vp(cs2) if want_cs2 else None, _stream()))
        return (out, cs2) if want_cs2 else out

    def destroy(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().pade_mlp_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def training_set(grid, closure, nsteps, every=1, max_samples=None, seed=0):
    """Run `grid` (an igrid with the dynamic procedure) for nsteps; every `every` steps
    collect the features of all points and the target Cs^2 = lambda(z) / Delta^2 of the
    plane they lie on.  Returns (X, y) CUDA tensors (float32)."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    dl = delta_les(grid.Lx / nx, grid.Ly / ny, grid.Lz / nz)
    Xs, ys = [], []
    for step in range(nsteps):
        grid.timeAdvance(use_graph=False)
        if (step + 1) % every:
            continue
        grads = [grid.field(f"duidxjC{i + 1}") for i in range(9)]
        X = closure.features(grads, dl, 1.0 / grid.Re)
        lam = torch.from_numpy(grid.info()["lambda"] / dl ** 2).to(X.device, torch.float32)
        y = lam[:, None].expand(nz, nx * ny).reshape(-1)  # point order (i, j, k), k slowest
        Xs.append(X)
        ys.append(y)
    X = torch.cat(Xs)
    y = torch.cat(ys)
    if max_samples is not None and X.shape[0] > max_samples:
        g = torch.Generator(device="cpu").manual_seed(seed)
        idx = torch.randperm(X.shape[0], generator=g)[:max_samples].to(X.device)
        X, y = X[idx].contiguous(), y[idx].contiguous()
    return X, y


def feature_range(X):
    """Per-feature minimum and maximum of a training set X (n x 10)."""
    return X.min(dim=0).values.cpu().numpy(), X.max(dim=0).values.cpu().numpy()


def train(closure, X, y, epochs=5, batch=4096, lr=2e-3, wd=0.0, seed=0, set_range=True):
    """Mini-batch AdamW over (X, y); returns the mean loss of each epoch.  set_range records
    the training set's feature range in the closure (its fallback test inside the LES)."""
    if set_range:
        closure.set_range(*feature_range(X))
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = X.shape[0]
    hist = []
    for _ in range(epochs):
        perm = torch.randperm(n, generator=g).to(X.device)
        tot = 0.0
        nb = 0
        for b0 in range(0, n - batch + 1, batch):
            idx = perm[b0:b0 + batch]
            tot += closure.train_step(X[idx].contiguous(), y[idx].contiguous(), lr, wd, want_loss=True)
            nb += 1
        hist.append(tot / max(nb, 1))
    return hist


def box_filter(f, r):
    """Mean over r x r x r blocks of a field held as a (nz, ny, nx) tensor (a Fortran array
    with reversed dimensions); every extent a multiple of r."""
    nz, ny, nx = f.shape
    return f.reshape(nz // r, r, ny // r, r, nx // r, r).mean(dim=(1, 3, 5))


def dns_training_set(n_dns=512, ratio=4, nsteps=60, snapshots=2, every=20, seed=5, kp=8.0, Re=1000.0,
                     cs2_max=0.25, max_samples=None):
    """Training pairs from a direct simulation (the a priori procedure): the solver without an
    SGS model on n_dns^3 from the seeded spectrum E(k) ~ k^4 exp(-2 (k/kp)^2), run nsteps
    steps; then `snapshots` times, `every` steps apart, its velocity is box-filtered by
    `ratio` onto the LES grid n_dns/ratio.  Targets: the local Smagorinsky coefficient that
    matches the resolved-to-subgrid energy flux of the filtered DNS,
        Cs^2 = max(0, -tau_ij S_ij) / (2 Delta^2 |S| S_ij S_ij),  tau_ij = <u_i u_j> - <u_i><u_j>
    (clipped to [0, cs2_max]), with S_ij and the features from the filtered field's gradients
    as the LES computes them (the filtered field passed through igrid's init sequence).
    Returns (X, y, info): CUDA float32 tensors and a dict of the run's figures."""
    from .IncompressibleGrid import igrid
    from .PadeDerOps import Pade6stagg
    from .synthetic import hit_initial_field_torch

    n_les = n_dns // ratio
    L_ = 2 * np.pi
    g = igrid()
    g.init(n_dns, n_dns, n_dns, Re=Re, useSGS=False)
    u, v, w = hit_initial_field_torch(n_dns, seed=seed, kp=kp)
    g.set_fields(u, v, w)
    del u, v, w
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        g.timeAdvance(use_graph=False)
        for _ in range(nsteps - 1):
            g.timeAdvance(use_graph=True)
    side.synchronize()
    les = igrid()
    les.init(n_les, n_les, n_les, Re=Re, useSGS=False)
    interp = Pade6stagg()
    L.check(interp.init(n_les, L_ / n_les, 1, True), "Pade6stagg.init")
    dl = delta_les(L_ / n_les, L_ / n_les, L_ / n_les)
    clo = LearnedClosure()
    Xs, ys = [], []
    for snap in range(snapshots):
        if snap:
            with torch.cuda.stream(side):
                for _ in range(every):
                    g.timeAdvance(use_graph=True)
            side.synchronize()
        uu = [g.field(nm) for nm in ("u", "v", "wC")]
        fu = [box_filter(a, ratio) for a in uu]
        tau = {}
        for i in range(3):
            for j in range(i, 3):
                tau[(i, j)] = box_filter(uu[i] * uu[j], ratio) - fu[i] * fu[j]
        del uu
        wE = torch.empty((n_les + 1, n_les, n_les), dtype=torch.float64, device="cuda")
        interp.interpz_C2E(fu[2].contiguous(), wE, 0, 0)
        les.set_fields(fu[0].contiguous(), fu[1].contiguous(), wE)
        grads = [les.field(f"duidxjC{i + 1}") for i in range(9)]
        G = [[grads[3 * i + j] for j in range(3)] for i in range(3)]  # G[i][j] = du_i/dx_j
        S = {(i, j): 0.5 * (G[i][j] + G[j][i]) for i in range(3) for j in range(i, 3)}
        w2 = {(i, j): (1.0 if i == j else 2.0) for (i, j) in S}
        SS = sum(w2[k] * S[k] * S[k] for k in S)
        Smag = torch.sqrt(2.0 * SS)
        flux = -sum(w2[k] * tau[k] * S[k] for k in S)
        den = 2.0 * dl * dl * Smag * SS
        cs2 = torch.where(den > 0, flux / torch.where(den > 0, den, torch.ones_like(den)), torch.zeros_like(den))
        cs2 = cs2.clamp(0.0, cs2_max)
        X = clo.features(grads, dl, 1.0 / Re)
        Xs.append(X)
        ys.append(cs2.reshape(-1).float())
        del tau, grads, G, S, SS, Smag, flux, den
    X = torch.cat(Xs)
    y = torch.cat(ys)
    info = {"n_dns": n_dns, "n_les": n_les, "steps": nsteps + every * (snapshots - 1), "tsim": g.info()["tsim"],
            "samples": int(X.shape[0]), "cs2_mean": float(y.mean()), "cs2_zero_fraction": float((y == 0).float().mean())}
    g.destroy()
    les.destroy()
    interp.destroy()
    clo.destroy()
    if max_samples is not None and X.shape[0] > max_samples:
        gen = torch.Generator(device="cpu").manual_seed(seed)
        idx = torch.randperm(X.shape[0], generator=gen)[:max_samples].to(X.device)
        X, y = X[idx].contiguous(), y[idx].contiguous()
    return X, y, info
