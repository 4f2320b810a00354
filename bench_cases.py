"""Single-kernel benchmark cases: one operation applied repeatedly to a device-resident
field (the driver of the Nsight Compute captures summarised under profiles/).

    python bench_cases.py --family cd10 --opcode 1 --dir 1 --n 256 --other 256 320 --repeat 3 --path df
    python bench_cases.py --family dense --opcode 1 --dir 1 --n 256 --other 256 256 --repeat 3
    python bench_cases.py --family dense --of cf90 --opcode 0 --dir 1 --n 256 --other 256 256 --repeat 3
    python bench_cases.py --family spectral --n 256 --repeat 3      # fft + ifft
    python bench_cases.py --family projection --n 256 --repeat 3
    python bench_cases.py --family les --n 128 --repeat 2           # TVD-RK3 steps
    python bench_cases.py --family les_learned --n 256 --repeat 1   # learned closure
    python bench_cases.py --family mlp --n 256 --repeat 5           # closure inference alone

Prints the mean CUDA-event time per application and the implied HBM throughput at
16 B/point (8 B/point for the FP32 path).  Not part of the library: a measurement tool
beside bench.py.
"""
import argparse
import os
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--family", default="cd10",
                    choices=["cd06", "cd10", "cf90", "gaussian", "stagg", "dense", "spectral", "projection", "les",
                             "les_learned", "mlp"])
    ap.add_argument("--opcode", type=int, default=1)
    ap.add_argument("--dir", type=int, default=1)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--other", type=int, nargs=2, default=[256, 320])
    ap.add_argument("--periodic", type=int, default=1)
    ap.add_argument("--bc", type=int, nargs=2, default=[0, 0])
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--path", default="df", choices=["df", "native", "fp32"])
    ap.add_argument("--of", default="cd10", choices=["cd10", "cf90"], help="operator of the dense family")
    a = ap.parse_args(argv)
    import torch

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import padeops_gb300 as P
    from padeops_gb300 import _lib as L
    from padeops_gb300 import build as B

    B.build()
    if a.family in ("spectral", "projection", "les", "les_learned"):
        return spectral_case(a, torch, P)
    if a.family == "dense":
        return dense_case(a, torch, P, L)
    if a.family == "mlp":
        return mlp_case(a, torch)
    path = {"df": L.PATH_DF, "native": L.PATH_NATIVE, "fp32": L.PATH_FP32}[a.path]
    dt = torch.float32 if path == L.PATH_FP32 else torch.float64
    n = a.n
    h = (2 * np.pi / n) if a.periodic else 1.0 / (n - 1)
    cls = {"cd06": P.cd06, "cd10": P.cd10, "cf90": P.cf90, "gaussian": P.gaussian, "stagg": P.cd06stagg}[a.family]
    o = cls()
    if a.family == "stagg":  # periodic cd06stagg; --opcode is the pade_apply stagg operation (0..7)
        rc = o.init(n, h) if a.periodic else o.init(n, h, True, True)
    else:
        rc = o.init(n, h, bool(a.periodic)) if a.family in ("cd06", "cd10") else o.init(n, bool(a.periodic))
    assert rc == 0, rc
    na, nb = a.other
    n_in, n_out = o.lengths(a.opcode)
    total = n * na * nb
    g = torch.Generator(device="cuda").manual_seed(0)
    f = torch.randn(n_in * na * nb, device="cuda", dtype=dt, generator=g)
    out = torch.empty(n_out * na * nb, device="cuda", dtype=dt)
    o.apply(a.opcode, a.dir, f, out, na, nb, a.bc[0], a.bc[1], path)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.repeat):
        o.apply(a.opcode, a.dir, f, out, na, nb, a.bc[0], a.bc[1], path)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.repeat
    bpp = 2 * f.element_size()
    print(f"{a.family} op{a.opcode} dir{a.dir} n={n} lines={na}x{nb} path={a.path}: {ms:.4f} ms/app, "
          f"{total / ms / 1e6:.1f} Gpts/s, {total * bpp / ms / 1e6:.1f} GB/s")


def dense_case(a, torch, P, L):
    """pade_dense_apply of a periodic cd10 operator (opcode 1 or 2) or the periodic cf90
    filter (opcode 0, residual form) along a.dir."""
    import ctypes

    n = a.n
    if a.of == "cf90":
        o = P.cf90()
        assert o.init(n, True) == 0
    else:
        o = P.cd10()
        assert o.init(n, 2 * np.pi / n, True) == 0
    na, nb = a.other
    total = n * na * nb
    g = torch.Generator(device="cuda").manual_seed(0)
    f = torch.randn(total, device="cuda", dtype=torch.float64, generator=g)
    out = torch.empty_like(f)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def run():
        L.check(L.lib().pade_dense_apply(o.handle, a.opcode, a.dir, ctypes.c_void_p(f.data_ptr()),
                                         ctypes.c_void_p(out.data_ptr()), na, nb, 0, 0, s), "dense_apply")

    ms = _timed(torch, run, a.repeat)
    print(f"dense {a.of} op{a.opcode} dir{a.dir} n={n} lines={na}x{nb}: {ms:.4f} ms/app, "
          f"{total / ms / 1e6:.1f} Gpts/s, {total * 16 / ms / 1e6:.1f} GB/s")


def mlp_case(a, torch):
    """Learned-closure inference (pade_mlp_infer_nu) on n^3 points of random gradients."""
    from padeops_gb300.sgs_learned import LearnedClosure, init_params

    n3 = a.n ** 3
    g = torch.Generator(device="cuda").manual_seed(0)
    grads = [torch.randn(n3, device="cuda", dtype=torch.float64, generator=g) for _ in range(9)]
    c = LearnedClosure(init_params(0))
    ms = _timed(torch, lambda: c.infer_nu(grads, 2 * np.pi / a.n, 1e-3), a.repeat)
    print(f"mlp inference n^3={n3}: {ms:.4f} ms/launch, {n3 * 80 / ms / 1e6:.1f} GB/s at 80 B/point")


def _timed(torch, fn, repeat):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(repeat):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / repeat


def spectral_case(a, torch, P):
    n = a.n
    d = 2 * np.pi / n
    g = torch.Generator(device="cuda").manual_seed(0)
    if a.family in ("les", "les_learned"):
        from padeops_gb300.synthetic import hit_initial_field

        u, v, w = hit_initial_field(n, seed=4)
        grid = P.igrid()
        if a.family == "les_learned":  # an untrained network: the cost does not depend on the weights
            from padeops_gb300.sgs_learned import LearnedClosure, init_params

            grid.init(n, n, n, learnedSGS=True, JudgeFreq=0)
            grid.set_mlp(LearnedClosure(init_params(0)))
        else:
            grid.init(n, n, n)
        dev = lambda x: torch.from_numpy(np.ascontiguousarray(x.T)).cuda()  # noqa: E731
        grid.set_fields(dev(u), dev(v), dev(w))
        ms = _timed(torch, lambda: grid.timeAdvance(use_graph=False), a.repeat)
        print(f"{a.family} n={n}: {ms:.3f} ms/step")
        return
    sp = P.spectral()
    sp.init(n, n, n, d, d)
    U = torch.randn((n, n, n // 2 + 1), dtype=torch.complex128, device="cuda", generator=g)
    if a.family == "spectral":
        f = torch.randn((n, n, n), dtype=torch.float64, device="cuda", generator=g)
        ms = _timed(torch, lambda: (sp.fft(f, U), sp.ifft(U, f)), a.repeat)
        print(f"spectral fft+ifft n={n}: {ms:.3f} ms")
        return
    po = P.padepoisson()
    po.init(d, d, d, sp)
    V = torch.randn_like(U)
    W = torch.randn((n + 1, n, n // 2 + 1), dtype=torch.complex128, device="cuda", generator=g)
    ms = _timed(torch, lambda: po.PressureProjection(U, V, W), a.repeat)
    print(f"projection n={n}: {ms:.3f} ms")


if __name__ == "__main__":
    main()
