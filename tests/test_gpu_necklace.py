"""GPU checks of the necklace quotient for Schur permanents of prime order.

The necklace kernel must give exactly the residues of the Glynn cofactor
path (itself checked against the oracle) and of the oracle, and the CRT of
its residues must reproduce the reference's published perm(S_n) table.
"""

import json

import pytest

import oracle
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _plan(n):
    # necklace moduli: primes == 1 (mod n) below 2^30
    from permgpu.crt import NECKLACE_PRIME_LIMIT, nth_root_of_unity, plan_schur
    primes, congruence, bound = plan_schur(n, NECKLACE_PRIME_LIMIT)
    return primes, [nth_root_of_unity(n, p) for p in primes], congruence, bound


@pytest.mark.parametrize("n", [3, 5, 7, 11, 13, 17, 19])
def test_necklace_matches_oracle(lib, n):
    from permgpu import _lib
    primes, omegas, _, _ = _plan(n)
    # extra moduli: small primes = 1 mod n and the trivial root omega = 1
    extra = [p for p in range(n + 1, 4000, n) if oracle._is_prime(p)][:3]
    ps = list(primes) + extra + extra[:1]
    ws = list(omegas) + [pow(2, (p - 1) // n, p) for p in extra] + [1]
    got = _lib.schur_residues(n, ps, ws, method="necklace")
    for p, w, r in zip(ps, ws, got):
        assert r == oracle.schur_mod_p(n, w, p, 8), (n, p, w)


@pytest.mark.parametrize("n", [23, 29])
def test_necklace_matches_glynn_cofactor_path(lib, n):
    from permgpu import _lib
    primes, omegas, _, _ = _plan(n)
    a = _lib.schur_residues(n, primes, omegas, method="necklace")
    b = _lib.schur_residues(n, primes, omegas, method="glynn")
    assert a == b


@pytest.mark.parametrize("n", [23, 29, 31, 37, 41, 43])
def test_schur_table_through_necklace(lib, n):
    # full-size property: the CRT of necklace residues is the published value
    from permgpu import _lib
    from permgpu.crt import crt
    table = json.loads((GOLDEN / "schur.json").read_text())["table"]
    primes, omegas, congruence, bound = _plan(n)
    res = _lib.schur_residues(n, primes, omegas, method="necklace")
    moduli = list(primes)
    if congruence:
        res.append(congruence[0])
        moduli.append(congruence[1])
    x = crt(res, moduli)
    m = 1
    for q in moduli:
        m *= q
    if x > bound:
        x -= m
    assert x == int(table[str(n)])


def test_auto_method_agrees_with_both_paths(lib):
    from permgpu import _lib
    from permgpu.crt import nth_root_of_unity, plan_schur
    for n in (19, 37):
        primes, omegas, _, _ = _plan(n)
        auto = _lib.schur_residues(n, primes, omegas)
        assert auto == _lib.schur_residues(n, primes, omegas, method="necklace")
        if n < 37:
            assert auto == _lib.schur_residues(n, primes, omegas, method="glynn")
    # a modulus above 2^30 takes the wide-modulus necklace kernel under
    # "auto" (n >= 37); it must agree with the Glynn minor
    primes = plan_schur(37)[0][:1] + [p for p in plan_schur(37, 1 << 31)[0][:1]]
    omegas = [nth_root_of_unity(37, p) for p in primes]
    assert _lib.schur_residues(37, primes, omegas)[1] == _lib.schur_residues(
        37, primes[1:], omegas[1:], method="glynn")[0]
    # the pinned residue of tests/test_cuda_device_schur_glynn.py:141-146
    assert _lib.schur_residues(33, [4294967161], [2662262]) == [1428739342]


def test_wide_necklace_matches_glynn_cofactor_path(lib):
    # odd moduli 2^30 <= p < 2^32 take the wide-modulus kernel (fully reduced
    # sums, 33-bit Montgomery step); the Glynn minor runs them through the
    # 32-bit (p < 2^31) and 64-bit (p >= 2^31) residue kernels
    from permgpu import _lib
    from permgpu.crt import nth_root_of_unity, plan_schur
    n = 37
    wide = plan_schur(n, 1 << 31)[0][:2] + plan_schur(n, 1 << 32)[0][:1]
    assert all(p >= 1 << 30 for p in wide) and wide[-1] > 1 << 31
    narrow = plan_schur(n)[0][:1]
    primes = narrow[:1] + wide[:1] + wide[1:]
    omegas = [nth_root_of_unity(n, p) for p in primes]
    a = _lib.schur_residues(n, primes, omegas, method="necklace")
    b = _lib.schur_residues(n, primes, omegas, method="glynn")
    assert a == b
    # narrow and wide moduli in one call come back in call order
    assert a[:1] == _lib.schur_residues(n, primes[:1], omegas[:1], method="necklace")
    assert a[1:] == _lib.schur_residues(n, primes[1:], omegas[1:], method="necklace")


@pytest.mark.parametrize("n", [41, 47])
def test_reference_gpu_residue_pins_through_wide_necklace(lib, n):
    # the reference's CUDA residues at 32-bit pseudo-Mersenne primes
    # (tests/test_cuda_device_schur_glynn.py:153-172), computed on the GPU
    from permgpu import _lib
    pins = [c for c in json.loads((GOLDEN / "schur.json").read_text())["pins"] if c["n"] == n]
    assert pins
    for pin in pins:
        assert _lib.schur_residues(n, [pin["p"]], [pin["omega"]]) == [pin["residue"]]
