"""GPU test of pg_exact_permanent_noalloc, the entry point for callers that
cannot allocate device memory: plug-ins whose host process owns every device
allocation through its own pool, and services that reserve a fixed memory
budget at start-up and must not grow it.  The entry point keeps its scratch
in a fixed 32 KiB array inside the library instead of calling cudaMalloc.

It must give exactly what the allocating entry point pg_exact_permanent
gives — integers, so the tolerance is zero — on two calls in a row (the
shared scratch keeps the previous call's contents and must be re-zeroed),
on the legacy default stream and on a stream the caller created, and it
must reject orders above 48 and output buffers too small for the bound.

Collected last (file name) so a failure here never hides the other tests;
it passes alone in a fresh process as well as after them.
"""

import ctypes
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PG_OK, PG_ERANGE, PG_EABORT, PG_EOVERFLOW = 0, 2, 5, 7


def _call(fn, a, limbs, *extra):
    a = np.ascontiguousarray(a, dtype=np.int64)
    out = np.zeros(limbs, dtype=np.uint32)
    st = fn(a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), a.shape[0],
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), limbs, *extra)
    return st, out


def _lib():
    from permgpu import _lib
    handle = _lib.load()
    assert handle.pg_cuda_runtime_available() == 1
    return _lib, handle


@pytest.mark.parametrize("n,seed,low,high", [(12, 1, -8, 8), (24, 0, -8, 8), (28, 7, -3, 3),
                                             (40, 300, 0, 1), (6, 2, -(1 << 20), 1 << 20)])
def test_noalloc_matches_allocating_entry_point_twice(n, seed, low, high):
    lib, h = _lib()
    rng = np.random.default_rng(seed)
    a = rng.integers(low, high + 1, (n, n), dtype=np.int64)
    limbs = lib.exact_limbs(a)
    st, want = _call(h.pg_exact_permanent, a, limbs)
    assert st == PG_OK, h.pg_last_error()
    for _ in range(2):
        st, got = _call(h.pg_exact_permanent_noalloc, a, limbs, None)
        assert st == PG_OK, h.pg_last_error()
        assert got.tolist() == want.tolist()


def test_noalloc_alternating_matrices_do_not_leak_state():
    lib, h = _lib()
    rng = np.random.default_rng(9)
    mats = [rng.integers(-8, 9, (20, 20), dtype=np.int64), rng.integers(-2, 3, (16, 16), dtype=np.int64)]
    want = [lib.exact_permanent(m, lib.exact_limbs(m)) for m in mats]
    for _ in range(2):
        for m, w in zip(mats, want):
            st, got = _call(h.pg_exact_permanent_noalloc, m, lib.exact_limbs(m), None)
            assert st == PG_OK
            assert lib.limbs_to_int(got) == w


def test_noalloc_on_a_caller_created_stream():
    import torch
    lib, h = _lib()
    rng = np.random.default_rng(11)
    a = rng.integers(-8, 9, (26, 26), dtype=np.int64)
    limbs = lib.exact_limbs(a)
    st, want = _call(h.pg_exact_permanent, a, limbs)
    assert st == PG_OK, h.pg_last_error()
    stream = torch.cuda.Stream()
    for _ in range(2):
        st, got = _call(h.pg_exact_permanent_noalloc, a, limbs, ctypes.c_void_p(stream.cuda_stream))
        assert st == PG_OK, h.pg_last_error()
        assert got.tolist() == want.tolist()


def test_noalloc_rejects_beyond_its_limits():
    lib, h = _lib()
    st, _ = _call(h.pg_exact_permanent_noalloc, np.ones((49, 49), np.int64), 16, None)
    assert st == PG_ERANGE
    assert b"2 <= n <= 48" in h.pg_last_error()
    st, _ = _call(h.pg_exact_permanent_noalloc, np.full((5, 5), 1 << 40, np.int64), 16, None)
    assert st == PG_EOVERFLOW
    # 12 x 12 entries in [-8, 8]: the bound needs more than one 32-bit limb
    a = np.random.default_rng(3).integers(-8, 9, (12, 12), dtype=np.int64)
    st, _ = _call(h.pg_exact_permanent_noalloc, a, 1, None)
    assert st == PG_ERANGE
    assert b"limb count" in h.pg_last_error()


def test_noalloc_stops_on_pg_abort_once_the_abort_word_exists():
    # pg_clear_abort creates the process's abort word (an allocation made
    # here by the test, not by the entry point); a 40 x 40 0/1 walk takes
    # seconds, and pg_abort from another host thread ends it early
    lib, h = _lib()
    h.pg_clear_abort()
    a = (np.random.default_rng(300).random((40, 40)) < 0.5).astype(np.int64)
    timer = threading.Timer(0.2, h.pg_abort)
    t0 = time.perf_counter()
    timer.start()
    try:
        st, _ = _call(h.pg_exact_permanent_noalloc, a, lib.exact_limbs(a), None)
    finally:
        timer.join()
        h.pg_clear_abort()
    assert st == PG_EABORT, h.pg_last_error()
    assert time.perf_counter() - t0 < 1.5
    # re-armed: the next call completes and agrees with the allocating path
    b = np.random.default_rng(5).integers(-8, 9, (18, 18), dtype=np.int64)
    st, got = _call(h.pg_exact_permanent_noalloc, b, lib.exact_limbs(b), None)
    assert st == PG_OK
    assert lib.limbs_to_int(got) == lib.exact_permanent(b, lib.exact_limbs(b))
