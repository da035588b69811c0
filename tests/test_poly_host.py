"""CPU: the polynomial API's validation, bounds and small cases (no GPU).

permgpu.poly mirrors rivin-perm's perm_polynomial.py public functions; the
argument checks and the certified bounds must match the reference's, and the
order-0/1 cases never touch the device."""

import pytest

from conftest import golden
from permgpu import poly


def test_bounds_match_reference():
    for c in golden("poly.json")["affine"]:
        assert poly.affine_permanent_bounds(c["constant"], c["linear"]) == \
            tuple(int(v) for v in c["bounds"])


def test_small_orders_need_no_device():
    assert poly.affine_permanent([], []) == (1,)
    assert poly.affine_permanent([[3]], [[-2]]) == (3, -2)
    assert poly.affine_permanent_mod([[3]], [[-2]], 7) == (3, 5)
    assert poly.affine_permanent_mod([], [], 9) == (1,)
    assert poly.rook_polynomial([]) == (1,)
    assert poly.rook_polynomial([[1]]) == (1, 1)
    assert poly.rook_polynomial([[0, 0], [0, 0]]) == (1, 0, 0)
    assert poly.weighted_rook_polynomial([[5]]) == (1, 5)
    assert poly.principal_permanent_polynomial([]) == (1,)


@pytest.mark.parametrize("call,error,message", [
    (lambda: poly.affine_permanent_mod([[1]], [[1]], 4), ValueError, "odd integer"),
    (lambda: poly.affine_permanent_mod([[1]], [[1]], 1), ValueError, "odd integer"),
    (lambda: poly.affine_permanent_mod([[1]], [[1]], (1 << 63) + 1), ValueError, "64-bit"),
    (lambda: poly.affine_permanent_mod([[1]], [[1]], True), TypeError, "integer"),
    (lambda: poly.affine_permanent_mod([[1]], [[1]], 3.0), TypeError, "integer"),
    (lambda: poly.affine_permanent([[1, 2]], [[1, 2]]), ValueError, "square"),
    (lambda: poly.affine_permanent([[1]], [[1, 0], [0, 1]]), ValueError, "same shape"),
    (lambda: poly.affine_permanent([[1.5]], [[1]]), TypeError, "integers"),
    (lambda: poly.affine_permanent([[0] * 64] * 64, [[0] * 64] * 64), ValueError, "less than 64"),
    (lambda: poly.affine_permanent([[1]], [[1]], parallel=1), TypeError, "boolean"),
    (lambda: poly.affine_permanent([[1]], [[1]], num_threads=-1), ValueError, "non-negative"),
    (lambda: poly.rook_polynomial([[2]]), ValueError, "0 or 1"),
    (lambda: poly.weighted_rook_polynomial([[-1]]), ValueError, "nonnegative"),
    (lambda: poly.affine_permanent([[1]], [[1]], backend="python"), ValueError, "GPU"),
])
def test_validation_matches_reference_contract(call, error, message):
    with pytest.raises(error, match=message):
        call()


def test_orders_beyond_the_reference_range_are_rejected():
    # the reference takes orders below 64 (perm_polynomial.py:151), and so
    # does the GPU engine; order 64 fails in validation, before any device
    a = [[1] * 64 for _ in range(64)]
    with pytest.raises(ValueError, match="less than 64"):
        poly.affine_permanent(a, a)
