"""GPU parity of the exact engine (pg_exact_permanent) and of the whole-call
API (permgpu.matrix_permanent / binary_permanent) against the reference's
exact values."""

import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu


def test_exact_golden_generic(lib):
    import permgpu
    from permgpu import workloads
    for c in golden("exact_generic.json")["cases"]:
        a = workloads.generic_matrix(c["n"], c["seed"], c["low"], c["high"])
        want = int(c["permanent"])
        assert permgpu.matrix_permanent(a.tolist(), method="generic") == want, c
        assert permgpu.matrix_permanent(a.tolist(), engine="residue") == want, c


def test_exact_generic32(lib):
    import permgpu
    from permgpu import workloads
    path = GOLDEN / "exact_generic32.json"
    want = int(json.loads(path.read_text())["permanent"])
    a = workloads.generic32()
    assert lib.exact_supported(a)
    assert permgpu.matrix_permanent(a.tolist(), method="generic") == want


@pytest.mark.parametrize("n", list(range(2, 27)))
def test_exact_vs_oracle_every_order(lib, n):
    rng = np.random.default_rng(50 + n)
    a = rng.integers(-8, 9, (n, n), dtype=np.int64)
    assert lib.exact_supported(a)
    assert lib.exact_permanent(a, lib.exact_limbs(a)) == oracle.exact_permanent(a.tolist())


@pytest.mark.parametrize("G", [3, 4, 5, 6])
def test_group_sizes_agree(lib, G):
    # entries sized so that exactly group size G is the largest that fits
    n = 26
    target = {3: 1000, 4: 180, 5: 60, 6: 30}[G]
    rng = np.random.default_rng(G)
    a = rng.integers(-1, 2, (n, n), dtype=np.int64) * (target // n + 1)
    a[:, 0] = target // 2
    assert lib.exact_permanent(a, lib.exact_limbs(a)) == oracle.exact_permanent(a.tolist())


@pytest.mark.parametrize("n", [24, 28, 32])
def test_float_row_form_and_its_fallback(lib, n):
    # entries in [-8, 8] take the float-row form at these orders (three rows
    # of every group of 4 as exact FP32 sums); half the rows with large
    # entries put two large rows in a group (three-row bound product above
    # 2^22, or groups of 3: integer form), and
    # rows of mixed bounds make the host put the largest row of each group
    # last.  Every result must equal the residue engine's at several primes.
    rng = np.random.default_rng(700 + n)
    primes = [2_147_483_647, 2_147_483_629, 1_000_000_007, 4_294_967_291]
    base = rng.integers(-8, 9, (n, n), dtype=np.int64)
    mixed = base.copy()
    mixed[::3] = rng.integers(-2, 3, (len(mixed[::3]), n))
    wide = base.copy()
    wide[::2] = rng.integers(-40, 41, (n // 2, n))
    for a in (base, mixed, wide):
        assert lib.exact_supported(a)
        v = lib.exact_permanent(a, lib.exact_limbs(a))
        assert lib.residues(a, primes) == [v % p for p in primes]


def test_exact_extremes(lib):
    # all-ones, negative identity, zero row, large entries near the limit
    for n in (5, 12, 20):
        assert lib.exact_permanent(np.ones((n, n), np.int64), 4) == \
            int(np.prod(np.arange(1, n + 1, dtype=object)))
        assert lib.exact_permanent(-np.eye(n, dtype=np.int64), 2) == (-1) ** n
        z = np.ones((n, n), np.int64)
        z[3] = 0
        assert lib.exact_permanent(z, 4) == 0
    big = np.random.default_rng(1).integers(-(1 << 24), 1 << 24, (6, 6), dtype=np.int64)
    assert lib.exact_permanent(big, lib.exact_limbs(big)) == oracle.exact_permanent(big.tolist())


def test_exact_rejects_out_of_range(lib):
    a = np.full((4, 4), 1 << 40, dtype=np.int64)
    assert not lib.exact_supported(a)
    with pytest.raises(lib.PermGpuError):
        lib.exact_permanent(a, 10)
    import permgpu
    assert permgpu.matrix_permanent(a.tolist()) == oracle.exact_permanent(a.tolist())


def test_binary_grid_exact(lib):
    import permgpu
    g = golden("binary.json")["grid_4x4x5_periodic01"]
    assert permgpu.binary_permanent(g["matrix"]) == int(g["permanent"])


def test_binary_cases_exact(lib):
    import permgpu
    for c in golden("binary.json")["cases"]:
        assert permgpu.binary_permanent(c["matrix"]) == int(c["permanent"])


def test_binary40_workload_at_full_size(lib):
    # The eight 40 x 40 Bernoulli(0.5) benchmark matrices (seeds 300..307)
    # through the whole binary API (matching blocks, exact engine) against
    # per(A) modulo two primes from pg_binary_residues: an independent
    # traversal whose residues are pinned to the reference's
    # binary_permanent_mod_p (perm_binary.py:943-1005, perm_binary_omp.c:
    # 236-347).  Each matrix is a full 2^39-state walk on both sides.
    import permgpu
    from permgpu import workloads
    primes = [2_147_483_647, 2_147_483_629]
    for m in workloads.binary40(8):
        v = permgpu.binary_permanent(m.tolist())
        assert v > 0
        assert lib.binary_residues(m, primes) == [v % p for p in primes]


def test_binary_residue_path_equals_exact_path(lib):
    import permgpu
    from permgpu.crt import binary_block_bound, binary_primes_above
    rng = np.random.default_rng(9)
    m = (rng.random((22, 22)) < 0.5).astype(np.uint8)
    exact = permgpu.binary_permanent(m.tolist())
    primes = binary_primes_above(binary_block_bound(m.tolist()))
    assert lib.binary_residues(m, primes) == [exact % p for p in primes]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_sharded_partials_combine_to_exact(lib, world):
    from permgpu import shard, workloads
    a = workloads.generic_matrix(24, 0)
    want = int(golden("exact_generic.json")["cases"][-1]["permanent"])
    words = [shard.exact_partial_words(a, *shard.state_range(24, r, world)) for r in range(world)]
    assert shard.combine_exact_words(words, 24) == want


@pytest.mark.parametrize("n", [40, 44, 48])
@pytest.mark.parametrize("kind", ["int", "binary"])
def test_exact_partial_windows_at_the_largest_orders(lib, n, kind):
    # a whole traversal at these orders takes minutes to hours; windows of
    # 2^22 Gray states at the start, the middle and the end check the exact
    # kernel's widest shapes (groups up to 10, two extra accumulator words)
    # against the oracle's unscaled range sum modulo two primes
    from permgpu import shard
    rng = np.random.default_rng(800 + n + (kind == "binary"))
    a = (rng.integers(-8, 9, (n, n)) if kind == "int"
         else (rng.random((n, n)) < 0.5).astype(np.int64))
    assert lib.exact_supported(a)
    states, w = 1 << (n - 1), 1 << 22
    for lo in (0, states // 2 + (1 << 24), states - w):
        v = shard.words_value(shard.exact_partial_words(a, lo, lo + w))
        for p in (2_147_483_647, 1_000_000_007):
            assert v % p == oracle.glynn_range_mod_p(a, p, lo, lo + w), (n, kind, lo, p)
