"""GPU parity of the residue engine (pg_residues / pg_schur_residues /
pg_binary_residues) against the reference's golden vectors and the oracle.

Bit-exact: every residue must equal the reference's.
"""

import itertools
import math
import random

import numpy as np
import pytest

import oracle
from conftest import golden

pytestmark = pytest.mark.gpu

INT64_MIN, INT64_MAX = -(1 << 63), (1 << 63) - 1


def _definition(matrix):
    n = len(matrix)
    return sum(math.prod(matrix[r][c] for r, c in enumerate(cols))
               for cols in itertools.permutations(range(n)))


def test_golden_residues_all_modulus_tiers(lib):
    for case in golden("generic_residues.json")["cases"]:
        m = np.array([[int(x) for x in r] for r in case["matrix"]], dtype=np.int64).reshape(
            len(case["matrix"]), len(case["matrix"]))
        assert lib.residues(m, case["moduli"]) == case["residues"], case["matrix"][:1]


@pytest.mark.parametrize("modulus", [1, 2, 9, 101, INT64_MAX])
def test_exhaustive_binary_matrices_through_order_three(lib, modulus):
    for order in range(1, 4):
        for entries in itertools.product((0, 1), repeat=order * order):
            m = [list(entries[r * order:(r + 1) * order]) for r in range(order)]
            assert lib.residues(np.array(m, dtype=np.int64), [modulus])[0] == \
                _definition(m) % modulus


def test_exhaustive_signed_order_two(lib):
    mods = [2, 3, 9, 15, 101, INT64_MAX]
    for entries in itertools.product((-1, 0, 1), repeat=4):
        m = [list(entries[:2]), list(entries[2:])]
        assert lib.residues(np.array(m, dtype=np.int64), mods) == \
            [_definition(m) % p for p in mods]


# odd moduli 2^31 <= m < 2^32 take the wide form of the 32-bit kernel:
# primes just above 2^31, 3037000501, the largest 32-bit prime, the
# reference's pseudo-Mersenne Schur primes and an odd composite
WIDE_MODULI = [2_147_483_659, 3_037_000_501, 4_294_966_153, 4_294_967_161,
               4_294_967_291, 4_294_967_295]


@pytest.mark.parametrize("n", [2, 3, 4, 5, 9, 16, 17, 22, 23])
def test_wide_32bit_moduli_against_oracle(lib, n):
    rng = np.random.default_rng(2000 + n)
    a = rng.integers(-(1 << 40), 1 << 40, (n, n), dtype=np.int64)
    want = [oracle.permanent_mod_p(a, p, 8) for p in WIDE_MODULI]
    assert lib.residues(a, WIDE_MODULI) == want
    # mixed with narrow and 64-bit moduli in one call, results in call order
    mods = [1_000_003] + WIDE_MODULI[:2] + [(1 << 61) - 1, 4_294_967_311]
    assert lib.residues(a, mods) == [oracle.permanent_mod_p(a, p, 8) for p in mods]


@pytest.mark.parametrize("n", [30, 34])
def test_wide_32bit_moduli_large_orders_against_exact(lib, n):
    # full-size property: residues equal the exact engine's integer mod m
    rng = np.random.default_rng(3000 + n)
    a = rng.integers(-2, 3, (n, n), dtype=np.int64)
    exact = lib.exact_permanent(a, 12)
    assert lib.residues(a, WIDE_MODULI) == [exact % p for p in WIDE_MODULI]


@pytest.mark.parametrize("n", [37, 40, 47, 55, 63])
def test_partial_windows_at_large_orders(lib, n):
    # a whole traversal above order 36 is too long here: windows of Gray
    # states at the start, the middle and the end run every kernel shape up
    # to 63 for narrow and wide 32-bit moduli against the oracle's range sum
    from permgpu import shard
    rng = np.random.default_rng(4000 + n)
    a = rng.integers(-(1 << 40), 1 << 40, (n, n), dtype=np.int64)
    mods = [2_147_483_647, 1_000_003, 4_294_967_291, 3_037_000_501]
    states, w = 1 << (n - 1), 1 << 20
    for lo in (0, states // 2 + (1 << 22), states - w):
        got = shard.residue_partials(a, lo, lo + w, mods)
        assert got == [oracle.glynn_range_mod_p(a, p, lo, lo + w) for p in mods], (n, lo)


def test_partial_residues_combine_to_the_whole(lib):
    from permgpu import shard
    rng = np.random.default_rng(4100)
    a = rng.integers(-50, 51, (21, 21), dtype=np.int64)
    mods = [2_147_483_647, 4_294_967_291]
    whole = lib.residues(a, mods)
    for world in (1, 3, 8):
        parts = [shard.residue_partials(a, *shard.state_range(21, r, world), mods)
                 for r in range(world)]
        for i, p in enumerate(mods):
            assert shard.combine_residues([q[i] for q in parts], p, 21) == whole[i]
    with pytest.raises(lib.PermGpuError, match="PG_EINVAL"):
        shard.residue_partials(a, 1, 8, mods)                 # odd bound
    with pytest.raises(lib.PermGpuError, match="PG_ERANGE"):
        shard.residue_partials(a, 0, 8, [(1 << 61) - 1])      # modulus >= 2^32


@pytest.mark.parametrize("n", list(range(2, 24)))
def test_every_small_order_against_oracle(lib, n):
    rng = np.random.default_rng(1000 + n)
    a = rng.integers(-(1 << 40), 1 << 40, (n, n), dtype=np.int64)
    mods = [3, 1_000_003, 2_147_483_647, 2_147_483_629, 1 << 20, 6, (1 << 61) - 1]
    want = [oracle.permanent_mod_p(a, p, 8) for p in mods]
    assert lib.residues(a, mods) == want


@pytest.mark.parametrize("n", [31, 33, 36])
def test_large_orders_compile_and_run(lib, n):
    # whole traversals: the identity has permanent 1 and a matrix with a zero
    # row permanent 0 mod every prime (orders above 36 are covered by the
    # partial windows of test_partial_windows_at_large_orders)
    a = np.eye(n, dtype=np.int64)
    assert lib.residues(a, [2_147_483_647, 1_000_003]) == [1, 1]
    a[n // 2, :] = 0
    assert lib.residues(a, [2_147_483_647]) == [0]


@pytest.mark.parametrize("domain", ["dense_signed", "binary", "sparse", "triangular", "rank_one",
                                    "repeated_rows", "zero_row", "block_diagonal"])
def test_structural_domains_and_symmetries(lib, domain):
    rng = random.Random(314159)
    order = 6
    m = [[rng.randrange(-5, 6) for _ in range(order)] for _ in range(order)]
    if domain == "binary":
        m = [[rng.randrange(2) for _ in range(order)] for _ in range(order)]
    elif domain == "sparse":
        m = [[v if rng.random() < 0.25 else 0 for v in r] for r in m]
    elif domain == "triangular":
        m = [[v if i <= j else 0 for j, v in enumerate(r)] for i, r in enumerate(m)]
    elif domain == "rank_one":
        m = [[(i - 2) * (j + 1) for j in range(order)] for i in range(order)]
    elif domain == "repeated_rows":
        m[-1] = m[0][:]
    elif domain == "zero_row":
        m[-1] = [0] * order
    elif domain == "block_diagonal":
        m = [[v if i // 3 == j // 3 else 0 for j, v in enumerate(r)] for i, r in enumerate(m)]
    want = _definition(m)
    for eq in (m, [list(r) for r in zip(*m)], [r[2:] + r[:2] for r in reversed(m)]):
        for p in (9, 101, INT64_MAX):
            assert lib.residues(np.array(eq, dtype=np.int64), [p])[0] == want % p


def test_many_moduli_one_launch(lib):
    from permgpu.crt import descending_primes
    a = np.random.default_rng(7).integers(-8, 9, (20, 20), dtype=np.int64)
    primes = descending_primes(1 << 600)          # ~20 primes < 2^31
    got = lib.residues(a, primes)
    exact = oracle.exact_permanent(a.tolist())
    assert got == [exact % p for p in primes]


def test_schur_golden_residues_and_pin(lib):
    s = golden("schur.json")
    for c in s["residues"]:
        assert lib.schur_residues(c["n"], [c["p"]], [c["omega"]])[0] == c["residue"], c
    # the n = 41 / 47 pins (32-bit primes) run through the wide-modulus
    # necklace kernel in test_gpu_necklace.py
    for pin in s["pins"]:
        if pin["n"] <= 33:
            assert lib.schur_residues(pin["n"], [pin["p"]], [pin["omega"]])[0] == pin["residue"]


def test_schur_exact_small_orders(lib):
    import permgpu
    table = golden("schur.json")["table"]
    for n in range(0, 24):
        want = 0 if n % 2 == 0 and n > 0 else (1 if n <= 1 else int(table[str(n)]))
        assert permgpu.permanent(n) == want


def test_schur_33_exact(lib):
    import permgpu
    assert permgpu.permanent(33) == int(golden("schur.json")["table"]["33"])


def test_binary_golden(lib):
    b = golden("binary.json")
    for c in b["cases"]:
        m = np.array(c["matrix"], dtype=np.uint8)
        for p, want in c.get("residues", {}).items():
            assert lib.binary_residues(m, [int(p)]) == [want]
    for c in b["bernoulli_residues"]:
        mat = (np.random.default_rng(c["seed"]).random((c["n"], c["n"])) < 0.5).astype(np.uint8)
        assert lib.binary_residues(mat, [c["p"]]) == [c["residue"]]


def test_binary_grid_residues(lib):
    g = golden("binary.json")["grid_4x4x5_periodic01"]
    m = np.array(g["matrix"], dtype=np.uint8)
    primes = [int(p) for p in g["residues"]]
    assert lib.binary_residues(m, primes) == [g["residues"][str(p)] for p in primes]


def test_binary_abi_rejections(lib):
    eye = np.eye(5, dtype=np.uint8)
    for p in (9, 5, 2):
        with pytest.raises(lib.PermGpuError):
            lib.binary_residues(eye, [p])
    bad = eye.copy()
    bad[0, 0] = 2
    with pytest.raises(lib.PermGpuError):
        lib.binary_residues(bad, [101])
    assert lib.binary_residues(eye, [101]) == [1]


def test_gpu_ext_drop_in(lib):
    from permgpu import BinaryGpuExt, GpuExt
    ext = GpuExt()
    assert ext.permanent_mod_p([[2, -1], [3, 4]], 101, 3) == 5
    rng = random.Random(271828 + 17)
    m = [[rng.randrange(-101, 101) for _ in range(17)] for _ in range(17)]
    assert ext.permanent_mod_p(m, 101) == oracle.permanent_mod_p(m, 101, 8)
    assert BinaryGpuExt().binary_permanent_mod_p([[1, 1], [1, 1]], 101) == 2
