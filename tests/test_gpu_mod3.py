"""GPU parity of the mod-3 engine (pg_permanent_mod3, pg_permanent_mod3_cols)
against the reference's mod-3 results, the oracle, and exact identities."""

import math

import numpy as np
import pytest

import oracle
from conftest import golden

pytestmark = pytest.mark.gpu


def test_reference_golden_cases(lib):
    from permgpu import mod3
    for c in golden("mod3.json")["cases"]:
        assert mod3.permanent_mod3_fast(c["matrix"]) == c["mod3"], len(c["matrix"])


@pytest.mark.parametrize("n", list(range(2, 25)))
def test_random_vs_oracle(lib, n):
    rng = np.random.default_rng(300 + n)
    a = rng.integers(-(1 << 62), 1 << 62, (n, n))
    assert lib.permanent_mod3(a) == oracle.permanent_mod_p(a, 3, 8)


def test_column_entry_matches_matrix_entry(lib):
    from permgpu import mod3
    rng = np.random.default_rng(9)
    for n in (3, 16, 31, 32, 33, 35):
        a = rng.integers(0, 3, (n, n))
        mags, sgns = mod3.encode_matrix_f3(a)
        assert lib.permanent_mod3_cols(mags, sgns, n) == lib.permanent_mod3(a)


def test_identities_up_to_order_40(lib):
    for n in (3, 20, 33, 40):
        assert lib.permanent_mod3(np.ones((n, n), np.int64)) == math.factorial(n) % 3
        assert lib.permanent_mod3(np.eye(n, dtype=np.int64)) == 1
        assert lib.permanent_mod3(2 * np.eye(n, dtype=np.int64)) == pow(2, n, 3)
        p = np.eye(n, dtype=np.int64)[np.random.default_rng(n).permutation(n)]
        assert lib.permanent_mod3(-p) == pow(2, n, 3)
