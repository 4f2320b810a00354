"""Restart files of the igrid LES (igrid.F90:2719-2802) on the GPU: a run dumped after 3
steps and read back into a fresh solver continues like the uninterrupted run."""
import os

import numpy as np
import pytest

import padeops_gb300 as P
from padeops_gb300.synthetic import hit_initial_field

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()


def test_restart_round_trip(tmp_path):
    n = 32
    u, v, w = hit_initial_field(n, seed=4)
    a = P.igrid()
    a.init(n, n, n)
    a.set_fields(_dev(u), _dev(v), _dev(w))
    for _ in range(3):
        a.timeAdvance(use_graph=False)
    step = a.dumpRestartFile(str(tmp_path), runID=1)
    assert step == 3
    for var, nz in (("u", n), ("v", n), ("w", n + 1)):
        assert os.path.getsize(tmp_path / f"RESTART_Run01_{var}.000003") == 8 * n * n * nz
    raw = np.fromfile(tmp_path / "RESTART_Run01_u.000003").reshape(n, n, n)  # (z, y, x): x fastest
    assert np.array_equal(raw, a.field("u").cpu().numpy())
    b = P.igrid()
    b.init(n, n, n)
    tsim = b.readRestartFile(str(tmp_path), 3, 1)
    ia, ib = a.info(), b.info()
    assert ib["step"] == 3
    # the info file keeps 5 significant digits (format g15.5): relative error up to ~1e-4
    assert abs(ib["tsim"] - ia["tsim"]) <= 1e-4 * ia["tsim"] and tsim == ib["tsim"]
    # the restored state equals the dumped one (set_fields re-projects a projected field)
    for var in ("u", "v", "w"):
        fa, fb = a.field(var), b.field(var)
        assert float((fa - fb).abs().max() / fa.abs().max()) < 1e-12, var
    for _ in range(2):
        a.timeAdvance(use_graph=False)
        b.timeAdvance(use_graph=False)
    for var in ("u", "v", "w"):
        fa, fb = a.field(var), b.field(var)
        assert float((fa - fb).abs().max() / fa.abs().max()) < 1e-10, var
    assert b.info()["step"] == 5
