"""Host-buffer calls above 8 MB run as a chunked copy/compute/copy pipeline (GPU).

Every line is computed by the same kernel arithmetic whichever chunk it falls in, so the
pipelined host-buffer result must equal the device-buffer result bit for bit, for lines
along x (contiguous runs), y (slabs) and z (pitched 2-D copies), real and complex.
"""
import numpy as np
import pytest

import padeops_gb300 as P

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev_result(obj, opcode, d, f, out_shape, bc):
    fd = torch.from_numpy(np.ascontiguousarray(f.T)).cuda()
    od = torch.empty(tuple(reversed(out_shape)), dtype=fd.dtype, device="cuda")
    na, nb = [s for k, s in enumerate(f.shape) if k != d - 1]
    obj.apply(opcode, d, fd, od, na, nb, *bc)
    torch.cuda.synchronize()
    return np.asfortranarray(od.cpu().numpy().T)


@pytest.mark.parametrize("d", [1, 2, 3])
@pytest.mark.parametrize("cplx", [False, True])
def test_pipelined_host_calls_equal_device_calls(d, cplx):
    n = 64
    shape = [128, 128, 128]
    shape[d - 1] = n  # 64 x 128 x 128 FP64 = 8.4 MB
    rng = np.random.default_rng(d + 10 * cplx)
    f = rng.standard_normal(shape)
    if cplx:
        f = f + 1j * rng.standard_normal(shape)
    f = np.asfortranarray(f)
    assert f.nbytes >= 8 << 20
    o = P.cd10()
    assert o.init(n, 1.0 / (n - 1), False) == 0
    na, nb = [s for k, s in enumerate(shape) if k != d - 1]
    for opcode, bc in ((1, (0, 0)), (2, (1, -1))):
        ref = _dev_result(o, opcode, d, f, shape, bc)
        out = np.zeros_like(f, order="F")
        o.apply(opcode, d, f, out, na, nb, *bc)
        assert np.array_equal(out, ref), (d, cplx, opcode)


def test_pipelined_named_entry_and_stagg_output_length():
    n = 128
    f = np.asfortranarray(np.random.default_rng(3).standard_normal((96, 96, n + 1)))
    st = P.cd06stagg()
    assert st.init(n, 1.0 / n) == 0
    out = np.zeros((96, 96, n), order="F")
    st.ddz_E2C(f, out, 96, 96)
    ref = _dev_result(st, 0, 3, f, (96, 96, n), (0, 0))
    assert np.array_equal(out, ref)
