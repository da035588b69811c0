"""Host-side abort of long launches: pg_abort() called from another host
thread while a multi-second traversal runs makes the call return PG_EABORT
within a fraction of a second (the kernels read the host-mapped abort word
once per 2^16 states, or per chunk, after each thread's first period);
pg_clear_abort() re-arms the library and
the next call computes the right value.  The failure is made on the host:
no kernel is broken, nothing waits on anything that is not set."""

import threading
import time

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _aborted_after(lib, fn, delay=0.2):
    timer = threading.Timer(delay, lib.load().pg_abort)
    t0 = time.perf_counter()
    timer.start()
    try:
        with pytest.raises(lib.PermGpuError) as err:
            fn()
    finally:
        timer.join()
        lib.load().pg_clear_abort()
    return err.value.status, time.perf_counter() - t0


def test_abort_exact_engine(lib):
    # 40 x 40 0/1 matrix: 2^39 Gray states, about 2.6 s uninterrupted
    a = (np.random.default_rng(301).random((40, 40)) < 0.5).astype(np.int64)
    lib.load().pg_clear_abort()
    status, took = _aborted_after(lib, lambda: lib.exact_permanent(a, lib.exact_limbs(a)))
    assert status == lib.PG_EABORT
    assert took < 1.5
    b = np.random.default_rng(7).integers(-8, 9, (20, 20), dtype=np.int64)
    assert lib.exact_permanent(b, lib.exact_limbs(b)) == oracle.exact_permanent(b.tolist())


def test_abort_residue_engine(lib):
    # one 31-bit prime over a 40 x 40 matrix: about 7 s uninterrupted
    a = np.random.default_rng(302).integers(-8, 9, (40, 40), dtype=np.int64)
    lib.load().pg_clear_abort()
    status, took = _aborted_after(lib, lambda: lib.residues(a, [2_147_483_647]))
    assert status == lib.PG_EABORT
    assert took < 1.5
    b = np.random.default_rng(8).integers(-8, 9, (16, 16), dtype=np.int64)
    p = 2_147_483_647
    assert lib.residues(b, [p]) == [oracle.exact_permanent(b.tolist()) % p]


def test_abort_batched_engine(lib):
    # 256 matrices of order 32, entries in [-3, 3]: about 2 s of one
    # persistent launch; its warps read the word once per 8 tasks
    mats = [np.random.default_rng(600 + i).integers(-3, 4, (32, 32), dtype=np.int64)
            for i in range(256)]
    lib.load().pg_clear_abort()
    status, took = _aborted_after(lib, lambda: lib.batch_exact(mats))
    assert status == lib.PG_EABORT
    assert took < 1.5
    small = [np.random.default_rng(700 + i).integers(-3, 4, (n, n), dtype=np.int64)
             for i, n in enumerate((12, 17, 21))]
    assert lib.batch_exact(small) == [oracle.exact_permanent(m.tolist()) for m in small]


def test_abort_flag_left_set_stops_the_next_launch_at_once(lib):
    # a raised word that nobody cleared makes every later long launch stop at
    # its first poll (after each thread's first 2^16 states: a 36 x 36 walk
    # gives every thread several hundred thousand); clearing it restores
    # normal service.  Launches too short for a poll complete as usual.
    a = np.random.default_rng(9).integers(-8, 9, (36, 36), dtype=np.int64)
    h = lib.load()
    h.pg_abort()
    try:
        t0 = time.perf_counter()
        with pytest.raises(lib.PermGpuError) as err:
            lib.exact_permanent(a, lib.exact_limbs(a))
        assert err.value.status == lib.PG_EABORT
        assert time.perf_counter() - t0 < 1.0
        b = np.random.default_rng(10).integers(-8, 9, (16, 16), dtype=np.int64)
        assert lib.exact_permanent(b, lib.exact_limbs(b)) == oracle.exact_permanent(b.tolist())
    finally:
        h.pg_clear_abort()
    c = np.random.default_rng(9).integers(-8, 9, (20, 20), dtype=np.int64)
    assert lib.exact_permanent(c, lib.exact_limbs(c)) == oracle.exact_permanent(c.tolist())
