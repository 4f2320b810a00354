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


def train(closure, X, y, epochs=5, batch=4096, lr=2e-3, wd=0.0, seed=0):
    """Mini-batch AdamW over (X, y); returns the mean loss of each epoch."""
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
