"""Run one compact operator repeatedly on a device-resident field (profiling driver).

    python -m padeops_gb300.profile_case --family cd10 --opcode 1 --dir 1 --n 256 \
        --other 256 320 --repeat 3 --path df

Used for Nsight Compute captures of a single kernel on a bounded case; prints the mean
CUDA-event time per application and the implied HBM throughput at 16 B/point.
"""
import argparse
import os
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--family", default="cd10", choices=["cd06", "cd10", "cf90", "gaussian"])
    ap.add_argument("--opcode", type=int, default=1)
    ap.add_argument("--dir", type=int, default=1)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--other", type=int, nargs=2, default=[256, 320])
    ap.add_argument("--periodic", type=int, default=1)
    ap.add_argument("--bc", type=int, nargs=2, default=[0, 0])
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--path", default="df", choices=["df", "native", "fp32"])
    a = ap.parse_args(argv)
    import torch

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import padeops_gb300 as P
    from padeops_gb300 import _lib as L
    from padeops_gb300 import build as B

    B.build()
    path = {"df": L.PATH_DF, "native": L.PATH_NATIVE, "fp32": L.PATH_FP32}[a.path]
    dt = torch.float32 if path == L.PATH_FP32 else torch.float64
    n = a.n
    h = (2 * np.pi / n) if a.periodic else 1.0 / (n - 1)
    cls = {"cd06": P.cd06, "cd10": P.cd10, "cf90": P.cf90, "gaussian": P.gaussian}[a.family]
    o = cls()
    rc = o.init(n, h, bool(a.periodic)) if a.family in ("cd06", "cd10") else o.init(n, bool(a.periodic))
    assert rc == 0, rc
    na, nb = a.other
    total = n * na * nb
    g = torch.Generator(device="cuda").manual_seed(0)
    f = torch.randn(total, device="cuda", dtype=dt, generator=g)
    out = torch.empty_like(f)
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


if __name__ == "__main__":
    main()
