"""CPU: the mod-3 engine's F_3 bit formulas, the oracle against the
reference's mod-3 results, and the API's validation (no GPU)."""

import numpy as np
import pytest

import oracle
from conftest import golden
from permgpu import mod3


def _val(m, s):
    return 0 if m == 0 else (1 if s == 0 else 2)


def test_bit_sliced_f3_formulas():
    # the row-sum update of csrc/pg_mod3.cu over every row-sum encoding (zero
    # has two) and every canonical column value
    def add(m1, s1, m2, s2):
        t = m1 ^ s1 ^ s2
        return (m2 & t) | (m1 ^ m2), (m2 & t) ^ s1

    def sub(m1, s1, m2, s2):
        t = s1 ^ s2
        return (m1 & t) | (m1 ^ m2), (m1 & t) ^ (m2 ^ s2)

    for m1 in (0, 1):
        for s1 in (0, 1):
            for m2, s2 in ((0, 0), (1, 0), (1, 1)):
                a, b = _val(m1, s1), _val(m2, s2)
                assert _val(*add(m1, s1, m2, s2)) == (a + b) % 3
                assert _val(*sub(m1, s1, m2, s2)) == (a - b) % 3


def test_oracle_matches_reference_mod3():
    for c in golden("mod3.json")["cases"]:
        if len(c["matrix"]) <= 26:
            assert oracle.permanent_mod_p(c["matrix"], 3, 8) == c["mod3"]
            assert oracle.permanent_mod3(c["matrix"]) == c["mod3"]


def test_encoding_and_small_cases():
    mags, sgns = mod3.encode_matrix_f3([[1, 2], [0, -1]])
    assert mags.tolist() == [0b01, 0b11] and sgns.tolist() == [0, 0b11]
    assert mod3.decode_f3_element(1, 1) == 2 and mod3.decode_f3_element(0, 1) == 0
    assert mod3.permanent_mod3_fast([]) == 1
    assert mod3.permanent_mod3_fast([[5]]) == 2


@pytest.mark.parametrize("matrix,error,message", [
    ([[7, 8]], ValueError, "square"),
    (np.empty((0, 2), dtype=np.int64), ValueError, "square"),
    ([[1.5]], TypeError, "integers"),
    (np.zeros((64, 64), dtype=np.int64), ValueError, "less than 64"),
])
def test_validation_matches_reference(matrix, error, message):
    with pytest.raises(error, match=message):
        mod3.permanent_mod3_fast(matrix)


def test_thread_argument_contract():
    with pytest.raises(ValueError, match="positive"):
        mod3.permanent_mod3_fast([[1]], num_threads=0)
    with pytest.raises(TypeError, match="positive integer"):
        mod3.permanent_mod3_fast([[1]], num_threads=True)
