"""Benchmark of the compact-operator hot path on GB300.

Workload (a "step"): CD10 first and second derivatives plus the CF90 compact filter along
x, y (periodic) and z (non-periodic, one-sided closures, bc 0) of a 256^3 FP64 field --
nine operator applications.  Fields are seeded random-mode sums (32 modes, |k_i| <= 64,
amplitudes N(0,1)|k|^-5/6, tanh(4(z-0.5)) profile in z), standing in for the reference's
data.  Metric: operator throughput in Gpts/s (points x operator applications per second).

  value     device throughput: inputs resident in HBM, CUDA events around K steps
  e2e       the same step through the reference-named C-ABI entry points with pinned
            HOST buffers (host->device copy, kernel, device->host copy per call)
  roofline  the fixed-stencil double-float line kernel (every launch of the step),
            algorithmic 16 B/point (read f once, write the result once) against the
            measured HBM copy bandwidth in MEASURED_PEAKS.json
  cpu_baseline  the oracle port of the reference algorithm on the host cores (OpenMP over
            lines), on the same workload

`extras` (same line): the FP32 and native-FP64 paths of the step, the tensor-core dense
(3xTF32) path for every operator of the step with its error against the FP64 path and its
speed-up, errors of the reduced-precision variants per wavenumber band, the 512^3 periodic
pressure projection, the 256^3 walled projection (with and without the Stokes pressure),
and the LES: s/step at 256^3 with the dynamic procedure and with the learned closure, and
the flow statistics (shell spectrum, kinetic energy, resolved and SGS dissipation) of
learned against dynamic runs at 256^3 (30 steps) and 64^3 (300 steps).

`--impl reference` times the oracle port alone (the Fortran reference cannot be built on
this hardware: no Fortran compiler or MPI) and prints its line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 256
NMODES, KMAX, SEED = 32, 64, 2
OPS = [("cd10 d1", 1), ("cd10 d2", 2), ("cf90", 0)]  # (name, opcode)
DIRS = (1, 2, 3)
BYTES_PER_POINT = 16  # FP64 read + write


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def make_field():
    from padeops_gb300.synthetic import random_modes

    return random_modes((N, N, N), NMODES, KMAX, SEED, z_nonperiodic=True, profile=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if len(r) >= 8 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 8 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) < 8:
                continue
            for nm, v in zip(names, r[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def setup_objects(P):
    dx = 2 * np.pi / N
    dz = 1.0 / (N - 1)
    cx = P.cd10()
    assert cx.init(N, dx, True) == 0
    cz = P.cd10()
    assert cz.init(N, dz, False) == 0
    fx = P.cf90()
    assert fx.init(N, True) == 0
    fz = P.cf90()
    assert fz.init(N, False) == 0
    return {("cd10", 1): cx, ("cd10", 2): cx, ("cd10", 3): cz, ("cf90", 1): fx, ("cf90", 2): fx, ("cf90", 3): fz}


def step_plan(objs):
    """The nine (object, opcode, dir) applications of one step."""
    plan = []
    for name, opc in OPS:
        fam = name.split()[0]
        for d in DIRS:
            plan.append((objs[(fam, d)], opc, d, f"{name} dir{d}"))
    return plan


def run_device(args, P, torch):
    dev = torch.device("cuda", torch.cuda.current_device())
    f_host = make_field()
    plan = step_plan(setup_objects(P))
    nops = len(plan)
    # one input and one output field per application: 2.4 GB per step >> L2 (no reuse)
    base = torch.from_numpy(np.ascontiguousarray(f_host.T)).to(dev)
    ins = [base.clone() for _ in range(nops)]
    outs = [torch.empty_like(base) for _ in range(nops)]
    del base
    stream = torch.cuda.current_stream(dev)
    npts = N ** 3

    def one_step(ev=None):
        for k, (obj, opc, d, _) in enumerate(plan):
            if ev is not None:
                ev[k][0].record(stream)
            obj.apply(opc, d, ins[k], outs[k], N, N, 0, 0)
            if ev is not None:
                ev[k][1].record(stream)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    # device-timed region (events on the launching stream) with per-launch events
    evs = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nops)]
           for _ in range(args.steps)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    from padeops_gb300.replicas import barrier

    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clk.start()
    torch.cuda.synchronize()
    barrier()
    t0.record(stream)
    for s in range(args.steps):
        one_step(evs[s])
    t1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = clk.stop()
    ms = t0.elapsed_time(t1)
    per_launch = np.zeros(nops)
    for s in range(args.steps):
        for k in range(nops):
            per_launch[k] += evs[s][k][0].elapsed_time(evs[s][k][1])
    per_launch /= args.steps
    del ins
    return ms / args.steps, per_launch, clocks, plan, f_host, outs


def run_e2e(args, P, torch, f_host):
    """Same step through the reference-named entry points with pinned host buffers."""
    objs = setup_objects(P)
    plan = step_plan(objs)
    host_in = torch.from_numpy(np.ascontiguousarray(f_host.T)).pin_memory()
    host_out = [torch.empty_like(host_in).pin_memory() for _ in range(3)]
    calls = []
    for k, (obj, opc, d, name) in enumerate(plan):
        fam = name.split()[0]
        out = host_out[k % 3]
        if fam == "cd10":
            fn = getattr(obj, ("dd" if opc == 1 else "d2d") + str(d))
            bc = (0, 0)
            calls.append(lambda fn=fn, out=out, bc=bc: fn(host_in, out, N, N, *bc))
        else:
            fn = getattr(obj, f"filter{d}")
            calls.append(lambda fn=fn, out=out: fn(host_in, out, N, N, 0, 0))
    for _ in range(max(1, args.warmup)):
        for c in calls:
            c()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(args.steps):
        for c in calls:
            c()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t) / args.steps
    nb = N ** 3 * 8 * len(calls)
    return dt, nb, nb


def cpu_baseline(args, f_host, steps=None):
    """The oracle port (reference algorithm; OpenMP over lines, y and z solves over blocks of
    consecutive lines as the reference's array-syntax SolveY / SolveZ) on the same workload."""
    from oracle import oracle as O

    O.build()
    dx = 2 * np.pi / N
    dz = 1.0 / (N - 1)
    work = []
    for name, opc in OPS:
        for d in DIRS:
            per = d != 3
            h = dx if per else dz
            if name.startswith("cd10"):
                work.append(lambda d=d, per=per, h=h, o=opc: O.cd10(f_host, h, periodic=per, order=o, dir=d))
            else:
                work.append(lambda d=d, per=per: O.cf90(f_host, periodic=per, dir=d))
    work[0]()  # warm-up (page-in)
    n = steps or 1
    t = time.perf_counter()
    for _ in range(n):
        results = [w() for w in work]
    dt = (time.perf_counter() - t) / n
    gpts = len(work) * N ** 3 / dt / 1e9
    return gpts, O.threads(), dt, results


def parity(plan, outs, oracle_out):
    """Normwise relative difference max|gpu - oracle| / max|oracle| of each application of
    the timed step (the outputs of its last step) against the oracle on the same field."""
    per = {}
    for (obj, opc, d, name), o, r in zip(plan, outs, oracle_out):
        g = o.cpu().numpy().T
        per[name] = float(np.abs(g - r).max() / np.abs(r).max())
    return max(per.values()), per


def _time(torch, fn, reps, stream=None):
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    st = stream or torch.cuda.current_stream()
    s.record(st)
    for _ in range(reps):
        fn()
    e.record(st)
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def band_errors(P, torch, lib, L, st):
    """Errors of the reduced-precision variants per wavenumber band, x lines of 256 points:
    line j carries one Fourier mode k_j = 1 + j mod 127 with a random phase; per line the
    max error is normalised by the line's max |double-float result|, then the max over the
    lines of each band k in [1, 32), [32, 64), [64, 96), [96, 128) is reported.  For the
    derivatives the double-float path's own error against the analytic derivative (the
    scheme's truncation error) is listed beside them."""
    import ctypes

    nl = 2048
    rng = np.random.default_rng(8)
    ks = 1 + (np.arange(nl) % (N // 2 - 1))
    ph = rng.uniform(0, 2 * np.pi, nl)
    x = np.arange(N) * 2 * np.pi / N
    arg = ks[:, None] * x[None, :] + ph[:, None]  # (line, point): x fastest in memory
    dev = torch.device("cuda", torch.cuda.current_device())
    f = torch.from_numpy(np.cos(arg)).to(dev)
    exact = {1: torch.from_numpy(-ks[:, None] * np.sin(arg)).to(dev),
             2: torch.from_numpy(-(ks[:, None] ** 2) * np.cos(arg)).to(dev)}
    bands = [(1, 32), (32, 64), (64, 96), (96, 128)]
    kt = torch.from_numpy(ks).to(dev)

    def per_band(err_line):
        return {f"k{lo}-{hi - 1}": float(err_line[(kt >= lo) & (kt < hi)].max()) for lo, hi in bands}

    res = {}
    h = 2 * np.pi / N
    for fam, opc, name in (("cd10", 1, "cd10 d1"), ("cd10", 2, "cd10 d2"), ("cf90", 0, "cf90")):
        o = P.cd10() if fam == "cd10" else P.cf90()
        assert (o.init(N, h, True) if fam == "cd10" else o.init(N, True)) == 0
        ref = torch.empty_like(f)
        o.apply(opc, 1, f, ref, nl, 1, 0, 0)
        got = torch.empty_like(f)
        L.check(lib.pade_dense_apply(o.handle, opc, 1, ctypes.c_void_p(f.data_ptr()),
                                     ctypes.c_void_p(got.data_ptr()), nl, 1, 0, 0, st))
        f32 = f.float().contiguous()
        o32 = torch.empty_like(f32)
        o.apply(opc, 1, f32, o32, nl, 1, 0, 0, P.PATH_FP32)
        torch.cuda.synchronize()
        scale = ref.abs().amax(dim=1)
        row = {"dense_tf32": per_band((got - ref).abs().amax(dim=1) / scale),
               "fp32_path": per_band((o32.double() - ref).abs().amax(dim=1) / scale)}
        if fam == "cd10":
            ex = exact[opc]
            row["fp64_path_vs_analytic"] = per_band((ref - ex).abs().amax(dim=1) / ex.abs().amax(dim=1))
        res[name] = row
    return res


def les_stats(stats, n):
    """Learned against dynamic after the same number of steps: spectrum deviation per shell
    (1 .. n/3), kinetic energy, resolved and SGS dissipation."""
    from padeops_gb300 import diagnostics as D

    d, lr = stats["dynamic"], stats["learned"]
    c = D.compare_spectra(lr["spectrum"], d["spectrum"], n, floor=1e-10)
    return {"steps": d["step"], "tsim": {"dynamic": d["tsim"], "learned": lr["tsim"]},
            "spectrum_max_rel_dev": c["max"], "spectrum_mean_rel_dev": c["mean"],
            "shells": f"1..{c['kmax']} (shells holding at least 1e-10 of the peak energy)",
            "spectrum_rel_dev_k1_4_8_16_32": [float(c["per_shell"][k - 1]) for k in (1, 4, 8, 16, 32)
                                              if k <= c["kmax"]],
            "ke": {"dynamic": d["ke"], "learned": lr["ke"]},
            "eps_resolved": {"dynamic": d["eps"][0], "learned": lr["eps"][0]},
            "eps_sgs": {"dynamic": d["eps"][1], "learned": lr["eps"][1]}}


def config1_extra(P, torch):
    """Config 1: CD06 periodic ddx / ddy / ddz (cd06%dd1..dd3) on the 64^3 field of 32 modes
    with |k_i| <= 16 (seed 1): errors against the oracle and the analytic derivative (the
    oracle's own error against it beside), CUDA-event time per call.  The 4 MB working set
    sits in L2, so the throughput is reported, not graded against HBM."""
    from oracle import oracle as O
    from padeops_gb300.synthetic import random_modes

    n = 64
    f, grad = random_modes(n, 32, 16, 1, gradient=True)
    dx = 2 * np.pi / n
    c = P.cd06()
    assert c.init(n, dx, True, 0, 0) == 0
    fd = torch.from_numpy(np.ascontiguousarray(f.T)).cuda()
    od = torch.empty_like(fd)
    res = {}
    for d, fn in ((1, c.dd1), (2, c.dd2), (3, c.dd3)):
        fn(fd, od, n, n)
        torch.cuda.synchronize()
        got = od.cpu().numpy().T
        ref = O.cd06(f, dx, periodic=True, dir=d)
        ex = grad[d - 1]
        sc = np.abs(ex).max()
        ms = _time(torch, lambda fn=fn: fn(fd, od, n, n), 50)
        t = time.perf_counter()
        O.cd06(f, dx, periodic=True, dir=d)
        ms_cpu = (time.perf_counter() - t) * 1e3
        res[f"dd{d}"] = {"relerr_vs_oracle": float(np.abs(got - ref).max() / np.abs(ref).max()),
                         "relerr_vs_analytic": float(np.abs(got - ex).max() / sc),
                         "oracle_relerr_vs_analytic": float(np.abs(ref - ex).max() / sc),
                         "ms": ms, "Gpts_s": n ** 3 / (ms * 1e-3) / 1e9, "oracle_ms": ms_cpu}
    return {"per_direction": res, "grid": [n, n, n],
            "field": "32 modes, integer |k_i| <= 16, amplitudes N(0,1)|k|^-5/6, random phases, seed 1",
            "note": "relerr normwise (max|a-b|/max|b|); the analytic error is CD06's truncation error at "
                    "k dx <= pi/2; 4 MB per field fits in L2 (throughput not roofline-graded)"}


def spectrum_velocity(torch, shape, kp, seed, dev):
    """Three physical fields with independent random phases and the spectrum
    E(k) ~ k^4 exp(-2 (k/kp)^2) (non-solenoidal): u_i = Re ifftn(sqrt(E/(4 pi k^2)) e^{i theta}),
    the real part being the Hermitian-symmetrised field; scaled to u_rms = 1."""
    nx, ny, nz = shape
    g = torch.Generator(device=dev).manual_seed(seed)
    kx = torch.fft.fftfreq(nx, 1.0 / nx, device=dev, dtype=torch.float64)
    ky = torch.fft.fftfreq(ny, 1.0 / ny, device=dev, dtype=torch.float64)
    kz = torch.fft.fftfreq(nz, 1.0 / nz, device=dev, dtype=torch.float64)
    # (z, y, x) tensor order = Fortran (x, y, z) memory order
    kk = torch.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    amp = torch.sqrt(kk ** 2 * torch.exp(-2.0 * (kk / kp) ** 2) / (4 * np.pi))
    del kk
    out = []
    for _ in range(3):
        th = torch.rand((nz, ny, nx), generator=g, device=dev, dtype=torch.float64) * (2 * np.pi)
        c = torch.polar(amp, th)
        del th
        out.append(torch.fft.ifftn(c).real.contiguous() * float(nx * ny * nz))
        del c
    rms = torch.sqrt(sum((x ** 2).mean() for x in out) / 3.0)
    return [x / rms for x in out]


def config3_fields(P, torch, shape, dev):
    """Config 3's spectral velocity on a grid of `shape`: uhat, vhat (nx/2+1, ny, nz) and what
    on the nz+1 edges, from the cell fields by spectral%fft and Pade6stagg%interpz_C2E
    (tests/test_PressureProj_PeriodicCD06.F90:66-83), fixOddball false."""
    nx, ny, nz = shape
    sp = P.spectral()
    sp.init(nx, ny, nz, 2 * np.pi / nx, 2 * np.pi / ny, fixOddball=False)
    u, v, wc = spectrum_velocity(torch, shape, 8.0, 3, dev)
    hs = (nz, ny, nx // 2 + 1)
    U = torch.empty(hs, dtype=torch.complex128, device=dev)
    V = torch.empty_like(U)
    WC = torch.empty_like(U)
    sp.fft(u, U)
    sp.fft(v, V)
    sp.fft(wc, WC)
    del u, v, wc
    st = P.cd06stagg()
    assert st.init(nz, 2 * np.pi / nz) == 0
    W = torch.empty((nz + 1, ny, nx // 2 + 1), dtype=torch.complex128, device=dev)
    st.InterpZ_C2E(WC, W, nx // 2 + 1, ny)
    del WC
    torch.cuda.synchronize()
    return sp, U, V, W


def config3_extra(P, torch, dev):
    """Config 3 (512^3 periodic, E(k) ~ k^4 exp(-2 (k/8)^2), non-solenoidal): max |div u| of
    the CD06 divergence before and after the projection, the projection's relative residual
    against the oracle (on a 512 x 512 x 64 slab of the same construction: the numpy oracle
    cannot hold 512^3 within the bench's time), and the transform and transpose times."""
    from oracle import spectral_oracle as SO
    from padeops_gb300 import decomp_2d as D

    res = {}
    n = 512
    d = 2 * np.pi / n
    sp, U, V, W = config3_fields(P, torch, (n, n, n), dev)
    po = P.padepoisson()
    po.init(d, d, d, sp)
    div = torch.empty((n, n, n), dtype=torch.float64, device=dev)
    po.DivergenceCheck(U, V, W, div)
    torch.cuda.synchronize()
    div0 = float(div.abs().max())
    U1, V1, W1 = U.clone(), V.clone(), W.clone()
    po.PressureProjection(U1, V1, W1)
    po.DivergenceCheck(U1, V1, W1, div)
    torch.cuda.synchronize()
    div1 = float(div.abs().max())
    umax = max(float(x.abs().max()) for x in (U1, V1, W1))
    ms_p = _time(torch, lambda: po.PressureProjection(U1, V1, W1), 3)
    ms_d = _time(torch, lambda: po.DivergenceCheck(U1, V1, W1, div), 3)
    phys = torch.empty((n, n, n), dtype=torch.float64, device=dev)
    ms_i = _time(torch, lambda: sp.ifft(U1, phys), 3)
    ms_f = _time(torch, lambda: sp.fft(phys, U1), 3)
    T = torch.empty_like(U)
    ms_t = _time(torch, lambda: (D.transpose_y_to_z(U, T), D.transpose_z_to_y(T, U)), 3)
    cbytes = 16 * (n // 2 + 1) * n * n
    res["grid_512"] = {
        "max_abs_div_before": div0, "max_abs_div_after": div1,
        "max_abs_div_after_rel": div1 / div0,
        "max_abs_velocity_hat": umax,
        "PressureProjection_ms": ms_p, "DivergenceCheck_ms": ms_d,
        "spectral_fft_ms": ms_f, "spectral_ifft_ms": ms_i,
        "fft_three_fields_ms": 3 * ms_f,
        "transpose_y_z_round_trip_ms": ms_t,
        "projection_compulsory_GBps": 6 * cbytes / (ms_p * 1e-3) / 1e9}
    del sp, po, U, V, W, U1, V1, W1, div, phys, T
    torch.cuda.empty_cache()
    # residual against the oracle on a slab of the same construction
    shape = (512, 512, 64)
    nx, ny, nz = shape
    sp, U, V, W = config3_fields(P, torch, shape, dev)
    uh, vh, wh = (np.asfortranarray(x.cpu().numpy().T) for x in (U, V, W))
    po = P.padepoisson()
    po.init(2 * np.pi / nx, 2 * np.pi / ny, 2 * np.pi / nz, sp)
    po.PressureProjection(U, V, W)
    div = torch.empty((nz, ny, nx), dtype=torch.float64, device=dev)
    po.DivergenceCheck(U, V, W, div)
    torch.cuda.synchronize()
    ref = SO.PeriodicPoisson(nx, ny, nz, 2 * np.pi / nx, 2 * np.pi / ny, 2 * np.pi / nz, fixOddball=False)
    ru, rv, rw, _ = ref.projection(uh, vh, wh)
    rdiv = ref.divergence(ru, rv, rw)

    def rel(t, r):
        return float(np.abs(t.cpu().numpy().T - r).max() / np.abs(r).max())

    res["slab_512x512x64"] = {"relerr_uhat": rel(U, ru), "relerr_vhat": rel(V, rv), "relerr_what": rel(W, rw),
                              "relerr_divergence_abs": float(np.abs(div.cpu().numpy().T - rdiv).max()
                                                             / max(np.abs(ru).max(), 1e-300)),
                              "max_abs_div_after": float(div.abs().max())}
    res["note"] = ("fixOddball false, w interpolated to the edges with the periodic CD06-stagg interpolation as in "
                   "tests/test_PressureProj_PeriodicCD06.F90; relerr normwise against the numpy/C oracle; one GPU "
                   "keeps one (i,j,k) layout, so the transposes are layout-preserving copies, timed for reference")
    del sp, po, U, V, W, div
    torch.cuda.empty_cache()
    return res


def extras(args, P, torch, f_host):
    """Secondary measurements of the other hot-path rows (rank 0): the FP32 and native-FP64
    paths of the same step, the 512^3 periodic projection, and the 256^3 LES step with the
    dynamic procedure and with the learned closure.  Errors are reported, not raised."""
    out = {}
    dev = torch.device("cuda", torch.cuda.current_device())
    plan = step_plan(setup_objects(P))
    npts = N ** 3
    reps = max(3, min(args.steps, 10))
    try:
        base = torch.from_numpy(np.ascontiguousarray(f_host.T)).to(dev)
        for path, dt, name, bpp in ((P.PATH_FP32, torch.float32, "fp32_path", 8),
                                    (P.PATH_NATIVE, torch.float64, "native_fp64_path", 16)):
            ins = [base.to(dt).clone() for _ in range(len(plan))]
            outs = [torch.empty_like(x) for x in ins]

            def step(ins=ins, outs=outs, path=path):
                for k, (obj, opc, d, _) in enumerate(plan):
                    obj.apply(opc, d, ins[k], outs[k], N, N, 0, 0, path)

            ms = _time(torch, step, reps if path == P.PATH_FP32 else 2)
            out[name] = {"value": len(plan) * npts / (ms * 1e-3) / 1e9, "unit": "Gpts/s", "ms_per_step": ms,
                         "achieved_GBps": len(plan) * npts * bpp / (ms * 1e-3) / 1e9, "bytes_per_point": bpp}
            del ins, outs
        del base
        torch.cuda.empty_cache()
    except Exception as ex:  # pragma: no cover - reported in the JSON line
        out["paths_error"] = repr(ex)
    try:
        import ctypes

        from padeops_gb300 import _lib as L

        lib = L.lib()
        base = torch.from_numpy(np.ascontiguousarray(f_host.T)).to(dev)
        ref = torch.empty_like(base)
        got = torch.empty_like(base)
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        xops = [(obj, opc, name) for (obj, opc, d, name) in plan if d == 1]
        # every operator of the step along its own direction (z non-periodic: bc 0, 0)
        per_op = {}
        for obj, opc, d, name in plan:
            obj.apply(opc, d, base, ref, N, N, 0, 0)
            L.check(lib.pade_dense_apply(obj.handle, opc, d, ctypes.c_void_p(base.data_ptr()),
                                         ctypes.c_void_p(got.data_ptr()), N, N, 0, 0, st))
            torch.cuda.synchronize()
            err = float((got - ref).abs().max() / ref.abs().max())

            def one_dense(obj=obj, opc=opc, d=d):
                lib.pade_dense_apply(obj.handle, opc, d, ctypes.c_void_p(base.data_ptr()),
                                     ctypes.c_void_p(got.data_ptr()), N, N, 0, 0, st)

            def one_line(obj=obj, opc=opc, d=d):
                obj.apply(opc, d, base, ref, N, N, 0, 0)

            md, ml = _time(torch, one_dense, reps), _time(torch, one_line, reps)
            per_op[name] = {"ms": md, "relerr_vs_fp64_path": err, "fp64_path_ms": ml, "speedup_vs_fp64_path": ml / md}
        ms = sum(v["ms"] for v in per_op.values())
        ms_line = sum(v["fp64_path_ms"] for v in per_op.values())
        xy = [v for k, v in per_op.items() if not k.endswith("dir3")]
        out["dense_tf32"] = {"value": len(plan) * npts / (ms * 1e-3) / 1e9, "unit": "Gpts/s",
                             "ms_per_step": ms, "speedup_vs_fp64_path_step": ms_line / ms,
                             "speedup_vs_fp64_path_xy": sum(v["fp64_path_ms"] for v in xy) / sum(v["ms"] for v in xy),
                             "achieved_GBps": len(plan) * npts * 16 / (ms * 1e-3) / 1e9,
                             "per_op": per_op,
                             "note": "tcgen05 kind::tf32, 3 products (hi/lo splits) of the dense A^-1 B; reduced "
                                     "precision; per-op CUDA-event times of the same 9 applications"}
        del base, ref, got
        torch.cuda.empty_cache()
        out["band_relerr"] = band_errors(P, torch, lib, L, st)
    except Exception as ex:  # pragma: no cover
        out["dense_error"] = repr(ex)
    try:
        out["config1_cd06_64"] = config1_extra(P, torch)
    except Exception as ex:  # pragma: no cover
        out["config1_error"] = repr(ex)
    try:
        out["projection_512"] = config3_extra(P, torch, dev)
    except Exception as ex:  # pragma: no cover
        out["projection_512_error"] = repr(ex)
    try:
        g = torch.Generator(device=dev).manual_seed(3)
        # walls at z = 0 and Lz (PeriodicInZ false), with and without the Stokes pressure, 256^3
        n = 256
        d = 2 * np.pi / n
        sp = P.spectral()
        sp.init(n, n, n, d, d)
        U = torch.randn((n, n, n // 2 + 1), dtype=torch.complex128, device=dev, generator=g)
        V = torch.randn_like(U)
        W = torch.randn((n + 1, n, n // 2 + 1), dtype=torch.complex128, device=dev, generator=g)
        wall = {}
        for stokes in (False, True):
            po = P.padepoisson()
            po.init(d, d, 1.0 / n, sp, PeriodicInZ=False, computeStokesPressure=stokes, Lz=1.0)
            wall["stokes" if stokes else "plain"] = _time(torch, lambda po=po: po.PressureProjection(U, V, W), 3)
            del po
        out["projection_wall_256"] = {"PressureProjection_ms": wall["plain"],
                                      "PressureProjection_stokes_ms": wall["stokes"],
                                      "note": "even/odd extension to 2 nz, library FFTs (double-float)"}
        del U, V, W, sp
        torch.cuda.empty_cache()
    except Exception as ex:  # pragma: no cover
        out["projection_error"] = repr(ex)
    try:
        from padeops_gb300.sgs_learned import LearnedClosure, dns_training_set, init_params, train
        from padeops_gb300.synthetic import hit_initial_field

        def tdev(a):
            return torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)

        from padeops_gb300 import diagnostics as D

        # training, a priori: a 512^3 direct simulation (no SGS model) from the config-3
        # spectrum E(k) ~ k^4 exp(-2 (k/8)^2), box-filtered to 128^3 at two times (4.2 M samples);
        # targets are the flux-matching Smagorinsky coefficients of the filtered DNS
        t0 = time.perf_counter()
        X, y, dinfo = dns_training_set(n_dns=512, ratio=4, nsteps=60, snapshots=2, every=20, seed=5, kp=8.0)
        t_dns = time.perf_counter() - t0
        clo = LearnedClosure(init_params(0))
        t0 = time.perf_counter()
        hist = train(clo, X, y, epochs=10, batch=4096, lr=3e-3)
        t_train = time.perf_counter() - t0
        nsamp = int(X.shape[0])
        del X, y
        torch.cuda.empty_cache()
        # the closure's inference kernel alone on 256^3 points (9 FP64 gradients in, nu out)
        n3 = 256 ** 3
        gen = torch.Generator(device=dev).manual_seed(11)
        grads = [torch.randn(n3, device=dev, dtype=torch.float64, generator=gen) for _ in range(9)]
        nu_buf = torch.empty(n3, device=dev, dtype=torch.float64)
        import ctypes as _ct

        from padeops_gb300 import _lib as _L
        from padeops_gb300.sgs_learned import _grads

        garr = _grads(grads)

        def infer_once():
            _L.check(_L.lib().pade_mlp_infer_nu(clo._h, garr, n3, 2 * np.pi / 256, 1e-3,
                                                _ct.c_void_p(nu_buf.data_ptr()), None,
                                                _ct.c_void_p(torch.cuda.current_stream().cuda_stream)))

        ms_inf = _time(torch, infer_once, 20)
        pk_gbs, pk_src = peaks()
        out["mlp_infer_256"] = {"ms_per_launch": ms_inf, "points": n3, "Gpts_s": n3 / ms_inf / 1e6,
                                "bytes_per_point": 80, "achieved_GBps": n3 * 80 / ms_inf / 1e6,
                                "frac_of_hbm_peak": n3 * 80 / ms_inf / 1e6 / pk_gbs,
                                "peak_source": pk_src,
                                "kernel": "k_mlp_infer_tc (tcgen05 kind::f16, BF16 operands, FP32 accumulation "
                                          "in tensor memory; GELU on BF16 pairs)"}
        del grads, nu_buf, garr
        torch.cuda.empty_cache()
        # developed flow: dynamic and learned (judged every 10 steps) from seed 5, 300 steps at 64^3
        n0, nrun = 64, 300
        u, v, w = hit_initial_field(n0, seed=5)
        st64 = {}
        judge64 = {}
        for mode in ("dynamic", "learned", "learned_planeavg", "learned_tol"):
            g1 = P.igrid()
            if mode != "dynamic":
                # learned_tol: the judge switches every point to lambda(z) while its error is above 0.25
                g1.init(n0, n0, n0, learnedSGS=True, JudgeFreq=10, learnedPlaneAvg=mode == "learned_planeavg",
                        JudgeTol=0.25 if mode == "learned_tol" else 0.0)
                g1.set_mlp(clo)
            else:
                g1.init(n0, n0, n0)
            g1.set_fields(tdev(u), tdev(v), tdev(w))
            while g1.info()["step"] < nrun:
                g1.timeAdvance(use_graph=False)
            inf = g1.info()
            st64[mode] = {"step": inf["step"], "tsim": inf["tsim"], "spectrum": D.energy_spectrum(g1),
                          "ke": D.kinetic_energy(g1), "eps": D.dissipation(g1, 1.0 / 1000.0)}
            if mode != "dynamic":
                j = g1.judge_info()
                judge64[mode] = {"last_judge_relerr": j["err"],
                                 "fallback_fraction": j["n_fallback"] / (3.0 * nrun * n0 ** 3)}
            del g1
        out["les_64_developed"] = {
            "pointwise": les_stats(st64, n0),
            "plane_averaged": les_stats({"dynamic": st64["dynamic"], "learned": st64["learned_planeavg"]}, n0),
            "judge_switch_tol_0.25": les_stats({"dynamic": st64["dynamic"], "learned": st64["learned_tol"]}, n0),
            "judge": judge64,
            "note": "closure trained a priori on the filtered 512^3 DNS; compared with the dynamic procedure from "
                    "seed 5 after 300 steps; judged every 10 steps (its lambda(z) the fallback outside the training "
                    "range); pointwise nu = Cs^2(x) Delta^2 |S|, plane_averaged nu = <Cs^2 Delta^2>_xy |S|; "
                    "judge_switch_tol_0.25: pointwise, with every point on lambda(z) while the judge's relative "
                    "difference exceeds 0.25"}
        n = 256
        nstat = 30  # steps from the same initial field before the statistics are compared
        u, v, w = hit_initial_field(n, seed=4)
        res, stats, judge = {}, {}, {}
        for mode in ("dynamic", "learned", "learned_judge10", "learned_planeavg", "constant"):
            g1 = P.igrid()
            if mode.startswith("learned"):
                g1.init(n, n, n, learnedSGS=True, JudgeFreq=10 if mode == "learned_judge10" else 0,
                        learnedPlaneAvg=mode == "learned_planeavg")
                g1.set_mlp(clo)
            elif mode == "constant":
                g1.init(n, n, n, DynamicProcedureType=0)
            else:
                g1.init(n, n, n)
            g1.set_fields(tdev(u), tdev(v), tdev(w))
            side = torch.cuda.Stream()
            with torch.cuda.stream(side):
                g1.timeAdvance(use_graph=False)  # step 0 carries the divergence check
                if mode == "learned_judge10":
                    # steps 1..10 eagerly (the judge steps cannot replay a fixed graph): one judge in ten
                    ms = _time(torch, lambda g1=g1: [g1.timeAdvance(use_graph=True) for _ in range(10)], 1,
                               stream=side) / 10.0
                else:
                    ms = _time(torch, lambda g1=g1: g1.timeAdvance(use_graph=True), 3, stream=side)
                while mode in ("dynamic", "learned", "learned_planeavg") and g1.info()["step"] < nstat:
                    g1.timeAdvance(use_graph=True)
            side.synchronize()
            res[mode] = ms
            if mode in ("dynamic", "learned", "learned_planeavg"):
                inf = g1.info()
                stats[mode] = {"step": inf["step"], "tsim": inf["tsim"], "spectrum": D.energy_spectrum(g1),
                               "ke": D.kinetic_energy(g1), "eps": D.dissipation(g1, 1.0 / 1000.0)}
            if mode == "learned_judge10":
                j = g1.judge_info()
                judge = {"last_judge_relerr": j["err"], "n_fallback": j["n_fallback"]}
            del g1
            torch.cuda.empty_cache()
        out["les_256"] = {"s_per_step_dynamic": res["dynamic"] / 1e3, "s_per_step_learned": res["learned"] / 1e3,
                          "learned_speedup": res["dynamic"] / res["learned"],
                          "s_per_step_learned_judge10": res["learned_judge10"] / 1e3,
                          "learned_judge10_speedup": res["dynamic"] / res["learned_judge10"],
                          "s_per_step_learned_planeavg": res["learned_planeavg"] / 1e3,
                          "learned_planeavg_speedup": res["dynamic"] / res["learned_planeavg"],
                          "s_per_step_constant_smagorinsky": res["constant"] / 1e3,
                          "speedup_bound_constant": res["dynamic"] / res["constant"],
                          "judge10": judge,
                          "config": "256^3 periodic, Re 1000, CFL 0.5, TVD-RK3, Smagorinsky (dynamic, deltaRatio 2) "
                                    "vs the learned closure; CUDA-graph steps (judged: 10 eager steps with one judge)",
                          "training": {"dns": dinfo, "dns_s": t_dns, "train_s": t_train, "samples": nsamp,
                                       "epochs": 10, "loss_first_last": [hist[0], hist[-1]]},
                          "statistics": les_stats(stats, n),
                          "statistics_planeavg": les_stats({"dynamic": stats["dynamic"],
                                                            "learned": stats["learned_planeavg"]}, n)}
    except Exception as ex:  # pragma: no cover
        out["les_error"] = repr(ex)
    return out


def traffic_per_launch():
    p = os.path.join(ROOT, "profiles", "line_kernel_traffic.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return d.get("dram_bytes_per_launch_256cubed")
        except Exception:
            return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the secondary measurements")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    metric = "CD10 d1+d2 and CF90 operator throughput, 256^3 FP64 (x,y periodic, z one-sided)"
    config = {"workload": "cd10 d1, cd10 d2, cf90 along x, y (periodic) and z (non-periodic, bc 0) on a "
                          "256^3 FP64 field; 9 operator applications per step",
              "grid": [N, N, N], "ops_per_step": 9, "fields": "seeded 32-mode sum, |k|<=64, tanh z profile",
              "l2": "each application reads its own 134 MB field and writes its own output (2.4 GB per step, "
                    "larger than the 126 MB L2); no flush needed",
              "parallelism": "replicas" if world > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        f_host = make_field()
        gpts, cores, dt, _ = cpu_baseline(args, f_host, steps=max(1, min(args.steps, 3)))
        line = {"metric": metric, "value": gpts, "unit": "Gpts/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config, "impl": "reference",
                "cpu_baseline": {"value": gpts, "unit": "Gpts/s", "cores": cores, "kind": "port",
                                 "sample": "full 256^3 step (9 applications), oracle C port with OpenMP over lines, "
                                           "y/z solves blocked over 16 consecutive lines"},
                "e2e": {"value": gpts, "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch

    import padeops_gb300 as P
    from padeops_gb300 import build as B

    B.build()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    ms_step, per_launch, clocks, plan, f_host, outs = run_device(args, P, torch)
    if world > 1:
        from padeops_gb300.replicas import max_over_ranks

        ms_step = max_over_ranks(ms_step, device="cuda")
    npts = N ** 3
    value = world * len(plan) * npts / (ms_step * 1e-3) / 1e9
    e2e = None
    if not args.no_e2e:
        dt, hb, db = run_e2e(args, P, torch, f_host)
        e2e = {"value": world * len(plan) * npts / dt / 1e9, "unit": "Gpts/s", "h2d_bytes_per_step": hb,
               "d2h_bytes_per_step": db}
    peak, src = peaks()
    t_kern = float(per_launch.sum())
    achieved = len(plan) * npts * BYTES_PER_POINT / (t_kern * 1e-3) / 1e9
    tr = traffic_per_launch()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": tr, "peak_source": src,
            "kernel": "k_lhalf (periodic lines, x and y) and k_lhalf_band (banded z): double-float chunked scans, "
                      "mean over the 9 launches",
            "algorithmic_bytes_per_launch": npts * BYTES_PER_POINT,
            "per_launch_ms": {p[3]: round(float(v), 4) for p, v in zip(plan, per_launch)}}
    cb = None
    par = None
    if rank == 0:
        gpts, cores, dt, oracle_out = cpu_baseline(args, f_host, steps=1)
        cb = {"value": gpts, "unit": "Gpts/s", "cores": cores, "kind": "port",
              "sample": "one full 256^3 step (9 applications), oracle C port with OpenMP over lines, "
                        "y/z solves blocked over 16 consecutive lines"}
        par = parity(plan, outs, oracle_out)
        del oracle_out
    del outs
    torch.cuda.empty_cache()
    ext = extras(args, P, torch, f_host) if (rank == 0 and not args.no_extras) else None
    if rank == 0:
        line = {"metric": metric, "value": value, "unit": "Gpts/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64 (double-float arithmetic)", "data": "synthetic",
                "config": config, "roofline": roof, "cpu_baseline": cb, "e2e": e2e, "clocks": clocks,
                "gpu_launches": len(plan) * args.steps,
                "parity_relerr": par[0], "parity_relerr_per_op": par[1],
                "parity_note": "outputs of the last timed step against the oracle on the same field, "
                               "max|gpu - oracle| / max|oracle| per application"}
        if ext is not None:
            line["extras"] = ext
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
