"""The multi-GPU form's host logic on CPU: two gloo ranks shard a job's
spins, combine their signal sums and take the slowest rank's time (the same
calls bench.py makes under torchrun)."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from dsim_gb300 import replicas
    lo, hi = replicas.shard(1001, rank, world)
    rng = np.random.default_rng(5)
    z = rng.standard_normal((1001, 2))          # per-spin m cos(phi), m sin(phi)
    comp = rng.integers(0, 4, 1001)
    local = np.zeros((5, 3))
    for c in range(-1, 4):
        sel = np.arange(lo, hi) if c < 0 else np.arange(lo, hi)[comp[lo:hi] == c]
        local[c + 1] = [z[sel, 0].sum(), z[sel, 1].sum(), len(sel)]
    total = replicas.combine_sums(local)
    t = replicas.max_time(0.5 + rank)
    q.put((rank, lo, hi, total, t))
    dist.destroy_process_group()


def test_two_rank_shards_and_reduction():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, lo0, hi0, t0, m0), (r1, lo1, hi1, t1, m1) = out
    assert (lo0, hi0, lo1, hi1) == (0, 501, 501, 1001)
    rng = np.random.default_rng(5)
    z = rng.standard_normal((1001, 2))
    comp = rng.integers(0, 4, 1001)
    want = np.zeros((5, 3))
    want[0] = [z[:, 0].sum(), z[:, 1].sum(), 1001]
    for c in range(4):
        want[c + 1] = [z[comp == c, 0].sum(), z[comp == c, 1].sum(), (comp == c).sum()]
    assert np.allclose(t0, want, rtol=1e-12) and np.array_equal(t0, t1)
    assert m0 == m1 == 1.5


def test_shard_covers_every_spin_once():
    from dsim_gb300.replicas import shard
    for n in (0, 1, 7, 1000, 1 << 20):
        for world in (1, 2, 3, 8):
            rs = [shard(n, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            assert max(h - l for l, h in rs) - min(h - l for l, h in rs) <= 1
