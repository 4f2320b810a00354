"""The oracle's blocked y/z path against its per-line path (CPU).

The oracle solves x lines one at a time and y / z lines in blocks of consecutive lines, each
statement over the whole block, as the reference's SolveY* / SolveZ* routines run their
statements over whole rows of lines.  Every line keeps its own operation order (no
contraction, no reassociation), so the blocked results must equal the per-line results bit
for bit: the same field, transposed so the direction becomes x, goes through the per-line
path.  Line counts that are not multiples of the block size leave a partial block.
"""
import itertools

import numpy as np
import pytest

from oracle import oracle as O

BCS = [0, 1, -1]


def _per_line(fn, f, dir, **kw):
    perm = {2: (1, 0, 2), 3: (2, 0, 1)}[dir]
    inv = np.argsort(perm)
    g = np.asfortranarray(f.transpose(perm))
    return fn(g, dir=1, **kw).transpose(inv)


def _field(shape, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal(shape))


@pytest.mark.parametrize("dir", [2, 3])
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("periodic,bc1,bcn", [(True, 0, 0)] + [(False, a, b) for a, b in itertools.product(BCS, BCS)])
def test_cd10_blocked_equals_per_line(dir, order, periodic, bc1, bcn):
    n = 40
    dx = 2 * np.pi / n if periodic else 1.0 / (n - 1)
    shape = [37, 5, 3]
    shape[dir - 1] = n
    f = _field(tuple(shape), 11 + order)
    kw = dict(periodic=periodic, bc1=bc1, bcn=bcn, order=order)
    got = O.cd10(f, dx, dir=dir, **kw)
    ref = _per_line(lambda g, dir, **k: O.cd10(g, dx, dir=dir, **k), f, dir, **kw)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("dir", [2, 3])
@pytest.mark.parametrize("periodic,bc1,bcn", [(True, 0, 0)] + [(False, a, b) for a, b in itertools.product(BCS, BCS)])
def test_cf90_blocked_equals_per_line(dir, periodic, bc1, bcn):
    n = 33
    shape = [21, 19, 4]
    shape[dir - 1] = n
    f = _field(tuple(shape), 5)
    kw = dict(periodic=periodic, bc1=bc1, bcn=bcn)
    got = O.cf90(f, dir=dir, **kw)
    ref = _per_line(lambda g, dir, **k: O.cf90(g, dir=dir, **k), f, dir, **kw)
    assert np.array_equal(got, ref)
