"""CPU: pin the C oracle against the reference's golden vectors.

The oracle (oracle/oracle_perm.c) is the checker for every GPU parity test;
these tests show it reproduces the reference exactly: residues across every
modulus tier, exact permanents, Schur residues and table values, binary
residues, and the reference's float code on small matrices.
"""

import math

import numpy as np
import pytest

import oracle
from conftest import golden


def test_generic_residues_match_reference_extension():
    for case in golden("generic_residues.json")["cases"]:
        m = [[int(x) for x in r] for r in case["matrix"]]
        for p, want in zip(case["moduli"], case["residues"]):
            if len(m) >= 16:
                assert oracle.permanent_mod_p(m, p, 4) == want
            else:
                assert oracle.permanent_mod_p(m, p, 1) == want


def test_exact_permanents_match_reference():
    from permgpu import workloads
    for case in golden("exact_generic.json")["cases"]:
        if case["n"] > 24:
            continue
        a = workloads.generic_matrix(case["n"], case["seed"], case["low"], case["high"])
        assert oracle.exact_permanent(a.tolist()) == int(case["permanent"])


def test_schur_residues_match_reference():
    for c in golden("schur.json")["residues"]:
        assert oracle.schur_mod_p(c["n"], c["omega"], c["p"], 4) == c["residue"]


def test_binary_residues_match_reference():
    b = golden("binary.json")
    for c in b["cases"]:
        for p, want in c.get("residues", {}).items():
            assert oracle.binary_mod_p(np.array(c["matrix"], dtype=np.uint8), int(p)) == want
    for c in b["bernoulli_residues"]:
        if c["n"] > 26:
            continue
        mat = (np.random.default_rng(c["seed"]).random((c["n"], c["n"])) < 0.5).astype(np.uint8)
        assert oracle.binary_mod_p(mat, c["p"], 8) == c["residue"]


def test_float_oracle_matches_reference_float_code():
    for c in golden("float_small.json")["cases"]:
        v, s = oracle.glynn_f64(c["matrix"], 1)
        assert abs(v - c["permanent"]) <= 1e-12 * max(1.0, s)


def test_complex_float_oracle_matches_reference_float_code():
    for c in golden("float_small.json")["complex_cases"]:
        a = np.array(c["re"]) + 1j * np.array(c["im"])
        v, s = oracle.glynn_c64(a)
        assert abs(v - complex(*c["permanent"])) <= 1e-12 * max(1.0, s)


def test_float_gradient_oracle_is_minor_permanent():
    rng = np.random.default_rng(3)
    a = rng.integers(-2, 3, (7, 7))
    g = oracle.glynn_f64_grad(a.astype(float), 2)
    for i in range(7):
        for j in range(7):
            minor = np.delete(np.delete(a, i, 0), j, 1)
            assert g[i, j] == oracle.exact_permanent(minor.tolist())


def test_oracle_against_reference_extension_when_built():
    c_ext, b_ext = oracle.reference_modules()
    if c_ext is None:
        pytest.skip("oracle/_ref not built (no reference checkout on this machine)")
    rng = np.random.default_rng(11)
    for n in (4, 9, 15, 18):
        a = rng.integers(-50, 51, (n, n))
        for p in (3, 9, 1_000_003, 2_147_483_647, 3_037_000_501, (1 << 62) + 135):
            assert oracle.permanent_mod_p(a, p, 2) == c_ext.permanent_mod_p(a.tolist(), p, 2)
    for n in (5, 9, 13):
        for p in (101, 1_000_003):
            if (p - 1) % n == 0:
                w = pow(2, (p - 1) // n, p)
                assert oracle.schur_mod_p(n, w, p) == c_ext.schur_permanent_mod_p(n, w, p, 1)
    m = (rng.random((14, 14)) < 0.5).astype(np.uint8)
    assert oracle.binary_mod_p(m, 2_147_483_647) == b_ext.binary_permanent_mod_p(
        m.tolist(), 2_147_483_647, 1)


def test_schur_table_small_orders_from_oracle_crt():
    # perm(S_n) = n * per(minor) reconstructed from oracle residues
    from permgpu.crt import crt, nth_root_of_unity, plan_schur
    table = golden("schur.json")["table"]
    for n in (3, 5, 7, 9, 11, 13, 15):
        primes, congruence, bound = plan_schur(n)
        res = [oracle.schur_mod_p(n, nth_root_of_unity(n, p), p) for p in primes]
        moduli = list(primes)
        if congruence:
            res.append(congruence[0])
            moduli.append(congruence[1])
        x = crt(res, moduli)
        if x > bound:
            x -= math.prod(moduli)
        assert x == int(table[str(n)])


def test_schur_table_agrees_with_reference_gpu_residue_pins():
    # the reference's CUDA residues for n = 33, 41, 47 (32-bit primes) are the
    # published perm(S_n) reduced mod those primes; the GPU tests check our
    # exact perm(S_n) against the same table
    s = golden("schur.json")
    for pin in s["pins"]:
        n, p, w = pin["n"], pin["p"], pin["omega"]
        assert pow(w, n, p) == 1
        assert int(s["table"][str(n)]) % p == pin["residue"]


def test_float_gradient_oracle_matches_reference_minors():
    # integer-valued 20x20: the reference's exact permanents of all 400
    # minors (perm.matrix_permanent) are the gradient
    data = golden("float20int_minors.json")
    c = data["cases"][0]
    a = np.array(c["matrix"], dtype=np.float64)
    g = oracle.glynn_f64_grad(a, 8)
    want = np.array([[float(int(x)) for x in row] for row in c["minors"]])
    assert np.array_equal(g, want)
    v, _ = oracle.glynn_f64(a, 8)
    assert v == float(int(c["permanent"]))


def test_affine_oracle_matches_reference_polynomial_engine():
    # oracle/oracle_perm.c or_affine_mod_p vs perm_polynomial (native engine)
    data = golden("poly.json")
    for c in data["affine"]:
        n = len(c["constant"])
        for m, want in zip(c["moduli"], c["residues"]):
            if n < 2:
                continue
            assert oracle.affine_mod_p(c["constant"], c["linear"], m) == want
        if n >= 2 and max(abs(v) for row in c["constant"] for v in row) < (1 << 40):
            assert oracle.affine_exact(c["constant"], c["linear"]) == [int(v) for v in c["exact"]]
    for c in data["principal"]:
        n = len(c["matrix"])
        eye = [[int(i == j) for j in range(n)] for i in range(n)]
        assert oracle.affine_mod_p(eye, c["matrix"], 1_000_003) == c["mod_1000003"]
