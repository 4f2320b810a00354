"""Two ranks on CPU (gloo): line sharding with no data collective reproduces the single
process result, and the timing reduction is the maximum over ranks."""
import os
import socket

import numpy as np
import pytest

from padeops_gb300.replicas import max_over_ranks, shard


def test_shard_covers_all_units():
    for n in (0, 1, 7, 64, 1000):
        for w in (1, 2, 3, 8):
            parts = [shard(n, r, w) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(w - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, f, out_path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O

    n1, n2, n = f.shape
    lines = n1 * n2
    lo, hi = shard(lines, rank, world)
    # z lines of a Fortran array: line l = (i, j) with l = i + n1 j
    flat = f.reshape(lines, n, order="F")
    mine = np.asfortranarray(flat[lo:hi].reshape(hi - lo, 1, n, order="F").transpose(1, 0, 2))
    res = O.cd10(mine, 1.0 / (n - 1), periodic=False, order=1, dir=3)
    np.save(f"{out_path}.{rank}.npy", res.reshape(hi - lo, n))
    m = max_over_ranks(10.0 + rank)
    np.save(f"{out_path}.{rank}.max.npy", np.array([m]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_line_sharding(tmp_path, oracle):
    import torch.multiprocessing as mp

    rng = np.random.default_rng(0)
    f = np.asfortranarray(rng.standard_normal((6, 5, 32)))
    out = str(tmp_path / "res")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, f, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = np.concatenate([np.load(f"{out}.{r}.npy") for r in range(2)])
    ref = oracle.cd10(f, 1.0 / 31, periodic=False, order=1, dir=3).reshape(30, 32, order="F")
    assert np.array_equal(got, ref)
    assert [float(np.load(f"{out}.{r}.max.npy")[0]) for r in range(2)] == [11.0, 11.0]
