"""Every periodic line kernel against the oracle (GPU).

Periodic lines of whole chunks have three kernels: the register-resident one
(reg_kernel.cuh), the shared-memory k_line (stencil_kernel.cuh) and the half-chunk k_lhalf
(half_kernel.cuh, on 32-row chunks or, for lines that are multiples of 16 rows, 16-row
chunks).  The library picks per path, operator and line (FP32: the register kernel;
double-float: the register kernel for tridiagonal operators along strided lines, k_lhalf
for the centred derivatives and cf90 where it applies, k_line otherwise), so the regular
parity tests see each kernel only on the cases it is picked for.  Here the periodic parity
tests run again with each choice forced (PADE_LINE_KERNEL = reg / shared / half,
PADE_HALF_CHUNK = 16; read once per process, so in a fresh process), at the same tolerances.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SELECT = ("cd06 or cd10_periodic or cf90 or stagg_periodic or fp32_path or bench_scale or range_free or "
          "periodic_whole_chunks or banded_whole_chunks")


@pytest.mark.parametrize("kernel", ["reg", "shared", "half", "half16"])
def test_periodic_parity_with_each_line_kernel(native_lib, kernel):
    env = dict(os.environ)
    if kernel == "half16":
        env["PADE_HALF_CHUNK"] = "16"
    else:
        env["PADE_LINE_KERNEL"] = kernel
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-p", "no:cacheprovider",
                        "tests/test_gpu_parity.py", "-k", SELECT],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
