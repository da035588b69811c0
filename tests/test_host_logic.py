"""CPU: host-side planning, preprocessing and drop-in validation (no GPU)."""

import math

import numpy as np
import pytest

from conftest import golden
from permgpu import crt
from permgpu import binary as pb
from permgpu.ext import BinaryGpuExt, GpuExt

INT64_MIN, INT64_MAX = -(1 << 63), (1 << 63) - 1


def test_graham_lehmer_matches_reference():
    for n, pair in golden("schur.json")["graham_lehmer"].items():
        got = crt.graham_lehmer_congruence(int(n))
        assert (list(got) if got else []) == pair


def test_schur_plan_covers_signed_range():
    for n in (3, 5, 9, 15, 21, 31, 33, 35, 41, 45, 47):
        primes, congruence, bound = crt.plan_schur(n)
        assert all(p < (1 << 31) and (p - 1) % n == 0 and crt.is_prime(p) for p in primes)
        product = math.prod(primes) * (congruence[1] if congruence else 1)
        assert product >= 2 * bound + 1
        # minimality: dropping the smallest prime loses coverage
        if primes:
            assert product // primes[-1] < 2 * bound + 1


def test_schur_plan_counts():
    # perm(S_33) needs 2 primes < 2^31 plus the theorem modulus; S_31 needs 3
    assert len(crt.plan_schur(33)[0]) == 2
    assert len(crt.plan_schur(31)[0]) == 3


def test_crt_and_sign_rule():
    primes = crt.descending_primes(10 ** 40)
    for v in (0, 1, -1, 12345678901234567890, -(10 ** 19) + 7):
        res = [v % p for p in primes]
        assert crt.signed_lift(res, primes, 10 ** 20) == v


def test_is_prime_matches_trial_division():
    for v in list(range(0, 2000)) + [2_147_483_647, 2_147_483_629, 3_037_000_499, 4_294_967_161]:
        want = v > 1 and all(v % d for d in range(2, math.isqrt(v) + 1))
        assert crt.is_prime(v) == want


def test_binary_bound_and_primes_match_reference_grid():
    g = golden("binary.json")["grid_4x4x5_periodic01"]
    bound = pb.binary_permanent_bound(g["matrix"])
    assert crt.binary_primes_above(bound) == g["reference_crt_primes"]
    assert bound >= int(g["permanent"])


def test_binary40_preprocessing_matches_reference():
    from permgpu import workloads
    ref = golden("binary.json")["binary40_preprocessing"]
    for mat, want in zip(workloads.binary40(8), ref):
        feasible, blocks = pb.matching_blocks(pb.row_masks(mat.tolist()))
        assert feasible == want["feasible"]
        assert sorted(len(b) for b in blocks) == want["block_sizes"]
        bits = [crt.binary_block_bound(b).bit_length() for b in blocks if len(b) > 1]
        assert bits == want["bound_bits"]


def test_matching_blocks_product_is_permanent():
    from oracle import exact_permanent
    rng = np.random.default_rng(5)
    for n in (3, 6, 9):
        for _ in range(20):
            m = (rng.random((n, n)) < 0.35).astype(int)
            feasible, blocks = pb.matching_blocks(pb.row_masks(m.tolist()))
            want = exact_permanent(m.tolist())
            got = math.prod(exact_permanent(b) for b in blocks) if feasible else 0
            assert got == want


@pytest.mark.parametrize(
    "matrix,modulus,threads,error,message",
    [
        (([1],), 101, 1, TypeError, "list of lists"),
        (1, 101, 1, TypeError, "list of lists"),
        ([(1,)], 101, 1, ValueError, "square"),
        ([[1, 2]], 101, 1, ValueError, "square"),
        ([[1], [2, 3]], 101, 1, ValueError, "square"),
        ([[0] * 64 for _ in range(64)], 101, 1, ValueError, "less than 64"),
        ([[1]], 0, 1, ValueError, "positive"),
        ([[1]], -3, 1, ValueError, "positive"),
        ([[1]], 1 << 63, 1, OverflowError, None),
        ([[1]], 101.0, 1, TypeError, None),
        ([[1.0]], 101, 1, TypeError, None),
        ([[1 << 63]], 101, 1, OverflowError, None),
        ([[INT64_MIN - 1]], 101, 1, OverflowError, None),
        ([[1]], 101, 1 << 31, OverflowError, None),
        ([[1]], 101, 1.0, TypeError, None),
    ],
)
def test_gpu_ext_validates_like_the_c_extension(matrix, modulus, threads, error, message):
    # identical table to the reference's tests/test_generic_native.py:206-233
    ext = GpuExt()
    for fn in (ext.permanent_mod_p, ext.ryser_permanent_mod_p):
        with pytest.raises(error, match=message):
            fn(matrix, modulus, threads)


def test_gpu_ext_empty_matrix_needs_no_device():
    assert GpuExt().permanent_mod_p([], 7) == 1
    assert GpuExt().permanent_mod_p([], 1) == 0
    assert GpuExt().schur_permanent_mod_p(1, 3, 7) == 1


def test_binary_ext_rejections():
    ext = BinaryGpuExt()
    eye = [[1, 0], [0, 1]]
    with pytest.raises(ValueError):
        ext.binary_permanent_mod_p(eye, 2)
    with pytest.raises(ValueError):
        ext.binary_permanent_mod_p(eye, 1)
    with pytest.raises(ValueError):
        ext.binary_permanent_mod_p([[1] * 64] * 64, 101)
    with pytest.raises(ValueError):
        ext.binary_permanent_mod_p([[2, 0], [0, 1]], 101)
    with pytest.raises(TypeError):
        ext.binary_permanent_mod_p(eye, 101.0)


def test_normalize_binary_strict():
    with pytest.raises(ValueError):
        pb.normalize_binary_matrix([[2]], strict=True)
    assert pb.normalize_binary_matrix([[2, 0], [0, -1]], strict=False) == ((1, 0), (0, 1))
    with pytest.raises(TypeError):
        pb.normalize_binary_matrix([[0.5]])


def _burnside_rotation_complement(length):
    # orbits of {0,1}^length under rotation and complement
    divisors = [d for d in range(1, length + 1) if length % d == 0]
    phi = lambda d: sum(1 for k in range(1, d + 1) if math.gcd(k, d) == 1)
    rot = sum(phi(d) * 2 ** (length // d) for d in divisors)
    comp = sum(phi(d) * 2 ** (length // d) for d in divisors if d % 2 == 0)
    return (rot + comp) // (2 * length)


def test_necklace_orbit_stats_match_reference():
    # the device walker, run on the host, against the reference's counts
    ext = GpuExt()
    for n, (reps, words) in golden("necklace_stats.json")["stats"].items():
        assert ext.schur_necklace_orbit_stats(int(n)) == (reps, words)
    for n in (3, 5, 7, 11, 13, 17, 19, 23):
        reps, words = ext.schur_necklace_orbit_stats(n)
        assert reps == _burnside_rotation_complement(n - 1) and words == 1 << (n - 1)
    for bad in (0, 2, 9, 25, 64):
        with pytest.raises(ValueError, match="odd prime"):
            ext.schur_necklace_orbit_stats(bad)


def test_schur_necklace_method_rejects_unsupported_inputs():
    from permgpu import _lib
    with pytest.raises(_lib.PermGpuError, match="PG_ERANGE"):
        _lib.schur_residues(9, [19], [pow(2, 2, 19)], method="necklace")       # n not prime
    with pytest.raises(_lib.PermGpuError, match="PG_ERANGE"):
        _lib.schur_residues(11, [4294967311], [1], method="necklace")          # p >= 2^30
    with pytest.raises(_lib.PermGpuError, match="PG_ERANGE"):
        _lib.schur_residues(11, [2147483629], [1], method="necklace")          # p >= 2^30
    with pytest.raises(_lib.PermGpuError, match="PG_ERANGE"):
        _lib.schur_residues(29, [2147483629], [1], method="necklace")          # no wide kernel
    with pytest.raises(_lib.PermGpuError, match="PG_ERANGE"):
        _lib.schur_residues(41, [4294967311], [1], method="necklace")          # p >= 2^32
    with pytest.raises(_lib.PermGpuError, match="PG_ERANGE"):
        _lib.schur_residues(11, [23], [5], method="necklace")                  # 5^11 != 1 mod 23
    with pytest.raises(ValueError):
        _lib.schur_residues(11, [23], [1], method="ryser")


def test_partial_residue_arguments_are_checked_on_the_host():
    # pg_residues_partial validates before any device call
    from permgpu import _lib, shard
    a = np.arange(16, dtype=np.int64).reshape(4, 4)
    for lo, hi, mods, code in [
            (1, 4, [1_000_003], "PG_EINVAL"),          # odd bound
            (4, 4, [1_000_003], "PG_ERANGE"),          # empty range
            (0, 16, [1_000_003], "PG_ERANGE"),         # beyond 2^(n-1) = 8
            (0, 4, [1 << 32], "PG_ERANGE"),            # modulus >= 2^32
            (0, 4, [4], "PG_ERANGE"),                  # even modulus
    ]:
        with pytest.raises(_lib.PermGpuError, match=code):
            shard.residue_partials(a, lo, hi, mods)
    with pytest.raises(_lib.PermGpuError, match="PG_ERANGE"):
        shard.residue_partials(np.ones((1, 1), dtype=np.int64), 0, 1, [7])   # n < 2


def test_fp64_entries_handle_orders_below_two_on_the_host():
    # n = 0 and n = 1 are answered without a device, like the reference's
    # empty-matrix and 1x1 conventions
    from permgpu import _lib
    per, grad, s = _lib.glynn_f64_fwd_bwd(np.array([[[2.5]], [[-1.0]]]))
    assert per.tolist() == [2.5, -1.0] and grad.ravel().tolist() == [1.0, 1.0]
    assert s.tolist() == [2.5, 1.0]
    per, s = _lib.glynn_c64(np.array([[[2.5 - 1j]], [[3j]]]))
    assert per.tolist() == [2.5 - 1j, 3j] and s[1] == 3.0
    per, s = _lib.glynn_c64(np.zeros((2, 0, 0), dtype=np.complex128))
    assert per.tolist() == [1, 1]
    with pytest.raises(_lib.PermGpuError, match="PG_ERANGE"):
        _lib.glynn_c64(np.zeros((1, 64, 64), dtype=np.complex128))


def test_matching_and_blocks_against_brute_force():
    # Hopcroft-Karp matching and the strongly-connected block split on every
    # kind of small 0/1 matrix: the matching is perfect whenever per(A) > 0,
    # absent when per(A) = 0, and the block permanents multiply to per(A)
    import itertools
    import random
    from permgpu import binary as pb

    def brute(a):
        k = len(a)
        return sum(all(a[i][p[i]] for i in range(k)) for p in itertools.permutations(range(k)))

    rng = random.Random(2024)
    for _ in range(1500):
        k = rng.randint(0, 7)
        dens = rng.random()
        a = [[1 if rng.random() < dens else 0 for _ in range(k)] for _ in range(k)]
        masks = pb.row_masks(a)
        want = brute(a)
        m = pb.perfect_matching(masks)
        if m is None:
            assert want == 0
        else:
            assert sorted(m) == list(range(k)) and all(a[r][m[r]] for r in range(k))
        feasible, blocks = pb.matching_blocks(masks)
        assert (math.prod(brute(b) for b in blocks) if feasible else 0) == want
        if feasible:
            assert sum(len(b) for b in blocks) == k
            assert all(brute(b) > 0 for b in blocks)
