"""Host-side pieces of oracle/ref_cuda.py (the harness that launches the
reference's own CUDA kernels) checked without a GPU: the Montgomery
constant, the 0/1 kernel's column orientation, the necklace frontier and
the Schur prime planner each against a direct computation of what the
reference's host code produces (perm_binary_cuda.cu:226-297,
perm_modp_cuda.cu:91-147, perm_cuda.py:289-404)."""

import itertools
import math

import numpy as np

import ref_cuda


def test_montgomery_negative_inverse():
    for p in (3, 65537, 1_000_000_007, 2_147_483_647):
        assert (p * ref_cuda._neg_inverse(p)) % (1 << 32) == (1 << 32) - 1


def test_orientation_lists_columns_by_size_with_the_densest_fixed():
    m = (np.random.default_rng(3).random((9, 9)) < 0.45).astype(np.uint8)
    m[np.arange(9), np.arange(9)] = 1
    offsets, rows, base, cost = ref_cuda._orientation(m, False)
    sizes = [int(m[:, c].sum()) for c in range(9)]
    fixed = sizes.index(max(sizes))
    variables = sorted((c for c in range(9) if c != fixed), key=lambda c: sizes[c])
    assert offsets == [0] + list(itertools.accumulate(sizes[c] for c in variables))
    assert rows == [r for c in variables for r in range(9) if m[r, c]]
    assert list(base[:9]) == [int(x) for x in m.sum(axis=1)]
    assert cost == sum(sizes[c] << (9 - 2 - b) for b, c in enumerate(variables))


def _prenecklace_prefixes(m, depth):
    # every length-`depth` prefix of a binary pre-necklace of length m with
    # at most m/2 ones, by brute force over words
    out = set()
    for word in range(1 << m):
        bits = [(word >> (m - 1 - i)) & 1 for i in range(m)]
        if sum(bits) > m // 2:
            continue
        rotations = [bits[i:] + bits[:i] for i in range(m)]
        if bits != min(rotations):
            continue
        out.add(tuple(bits[:depth]))
    return out


def test_necklace_frontier_covers_every_necklace_prefix():
    m, depth = 12, 7
    tasks = ref_cuda.necklace_frontier(m, depth)
    prefixes = {tuple(((int(t["word"]) >> (m - 1 - i)) & 1) for i in range(depth)) for t in tasks}
    assert _prenecklace_prefixes(m, depth) <= prefixes
    assert all(int(t["weight"]) == bin(int(t["word"])).count("1") for t in tasks)
    assert all(int(t["word"]) % (1 << (m - depth)) == 0 for t in tasks)


def test_schur_gpu_primes_cover_the_bound():
    for n in (41, 47):
        primes, cong = ref_cuda.schur_gpu_primes(n)
        assert all(q % n == 1 and q < (1 << 32) for q in primes)
        assert primes == sorted(primes, reverse=True)
        bound = math.isqrt(n ** n) + 1
        assert math.prod(primes) * cong[1] >= 2 * bound + 1
        assert math.prod(primes[:-1]) * cong[1] < 2 * bound + 1
