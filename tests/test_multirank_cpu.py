"""CPU, world_size 2 (gloo): the multi-rank path with no GPU.

Ranks split the Gray states with permgpu.shard.state_range, compute their
partial Glynn sums (here with the CPU oracle standing in for each rank's
GPU), exchange them with a gloo collective and combine on the host.  The
combined value must equal the oracle's full result.  bench.py's barrier and
max-over-ranks helpers are exercised on the same process group.
"""

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _exact_partial_python(a, lo, hi):
    """Unscaled exact Glynn sum over Gray states [lo, hi) (Python ints)."""
    n = len(a)
    g = lo ^ (lo >> 1)
    s = [sum(-a[i][j] if (j < n - 1 and (g >> j) & 1) else a[i][j] for j in range(n))
         for i in range(n)]
    total = 0
    for st in range(lo, hi):
        if st != lo:
            j = (st & -st).bit_length() - 1
            sub = ((st >> (j + 1)) & 1) == 0
            for i in range(n):
                s[i] += -2 * a[i][j] if sub else 2 * a[i][j]
        prod = 1
        for v in s:
            prod *= v
        total += -prod if st & 1 else prod
    return total


def _worker(rank, world, port, q):
    sys.path.insert(0, str(ROOT / "rivin-perm_gb300"))
    sys.path.insert(0, str(ROOT / "oracle"))
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world))
    import numpy as np
    import torch
    import torch.distributed as dist
    import oracle
    from permgpu import shard
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a = np.random.default_rng(17).integers(-5, 6, (11, 11)).tolist()
        n = len(a)
        p = 1_000_003
        lo, hi = shard.state_range(n, rank, world, align=64)
        # residue partials
        part = oracle.glynn_range_mod_p(a, p, lo, hi, 1)
        t = torch.tensor([part], dtype=torch.int64)
        gathered = [torch.zeros_like(t) for _ in range(world)]
        dist.all_gather(gathered, t)
        res = shard.combine_residues([int(x.item()) for x in gathered], p, n)
        # exact partials as words (as the GPU engine returns them)
        S = _exact_partial_python(a, lo, hi)
        words = [(S >> (32 * w)) & 0xffffffff for w in range(8)]
        words[-1] = S >> (32 * 7)          # signed top word
        wt = torch.tensor(words, dtype=torch.int64)
        wl = [torch.zeros_like(wt) for _ in range(world)]
        dist.all_gather(wl, wt)
        exact = shard.combine_exact_words([w.tolist() for w in wl], n)
        # the single-permanent split of bench.py's split workload: the same
        # product function, with the Python partial standing in for the
        # rank's GPU and the torch.distributed gather over gloo
        def stand_in(m, lo_, hi_):
            S_ = _exact_partial_python(m, lo_, hi_)
            w = [(S_ >> (32 * k)) & 0xffffffff for k in range(8)]
            w[-1] = S_ >> (32 * 7)
            return w
        split = shard.split_exact_permanent(a, rank, world, partial=stand_in)
        bench.barrier(world)
        mx = bench.max_over_ranks(world, float(rank + 1))
        if rank == 0:
            q.put((res, exact, mx, oracle.permanent_mod_p(a, p, 1), oracle.exact_permanent(a),
                   split))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharded_glynn_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
        assert p.exitcode == 0
    res, exact, mx, want_res, want_exact, split = q.get(timeout=10)
    assert res == want_res
    assert exact == want_exact
    assert split == want_exact
    assert mx == 2.0


def test_state_ranges_partition_the_walk():
    sys.path.insert(0, str(ROOT / "rivin-perm_gb300"))
    from permgpu import shard
    for n in (2, 5, 12, 20):
        for world in (1, 2, 3, 7):
            ranges = [shard.state_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == 1 << (n - 1)
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c
