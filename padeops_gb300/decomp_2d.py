"""Pencil transposes of 2DECOMP&FFT (transpose_x_to_y, _y_to_z, _z_to_y, _y_to_x) for one GPU.

With a single rank the x, y and z pencils all hold the full (nx, ny, nz) grid in the same
(i, j, k) Fortran order, so each transpose is a device-to-device copy
(``pade_transpose``).  src and dst are CUDA tensors of float64 or complex128.
"""
from . import _lib as L
from ._base import buffer


def _t(frm, to, src, dst):
    ps, cs, s, ns = buffer(src, "src", complex_ok=True)
    pd, cd, _, nd = buffer(dst, "dst", complex_ok=True)
    if s is None:
        raise TypeError("src must be a CUDA tensor")
    if cs != cd or ns != nd:
        raise ValueError("src and dst must have the same size and type")
    n = ns // 2 if cs else ns
    L.check(L.lib().pade_transpose(frm, to, ps, pd, n, 1, 1, 16 if cs else 8, s), "transpose")


def transpose_x_to_y(src, dst, decomp=None):
    _t(1, 2, src, dst)


def transpose_y_to_z(src, dst, decomp=None):
    _t(2, 3, src, dst)


def transpose_z_to_y(src, dst, decomp=None):
    _t(3, 2, src, dst)


def transpose_y_to_x(src, dst, decomp=None):
    _t(2, 1, src, dst)
