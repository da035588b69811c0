"""GPU parity of the batched engine (pg_batch_*) against the per-matrix
exact path and the oracle, including uneven orders, tiny and external
matrices, and every tuning candidate."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _mixed_batch():
    rng = np.random.default_rng(123)
    mats = [np.zeros((0, 0), np.int64), np.array([[-7]], np.int64)]
    for n in list(range(2, 23)) + [5, 9, 2, 17, 3]:
        mats.append(rng.integers(-3, 4, (n, n), dtype=np.int64))
    mats.append(rng.integers(-8, 9, (12, 12), dtype=np.int64) * 1000)   # G < 4 -> external
    mats.append(np.ones((34, 34), np.int64)[:6, :6])
    return mats


def test_mixed_batch_matches_oracle(lib):
    from permgpu.batch import batch_permanents
    mats = _mixed_batch()
    got = batch_permanents(mats, tune=None)
    want = [oracle.exact_permanent(m.tolist()) for m in mats]
    assert got == want


def test_batch4096_prefix_matches_per_matrix_path(lib):
    from permgpu import workloads
    mats = workloads.batch4096()[:512]
    plan = lib.BatchPlan(mats)
    plan.launch()
    got = plan.results()
    plan.close()
    for m, v in zip(mats, got):
        assert v == lib.exact_permanent(m, lib.exact_limbs(m))
    small = [(m, v) for m, v in zip(mats, got) if m.shape[0] <= 16][:40]
    for m, v in small:
        assert v == oracle.exact_permanent(m.tolist())


@pytest.mark.parametrize("tune", [(13, 6, 2), (11, 5, 1), (15, 8, 2), (9, 3, 2)])
def test_tuning_does_not_change_results(lib, tune):
    from permgpu import workloads
    mats = workloads.batch4096(count=200, seed=44)
    base = lib.batch_exact(mats)
    plan = lib.BatchPlan(mats, tune)
    for _ in range(2):                 # graph replays reset their state
        plan.launch()
        assert plan.results() == base
    plan.close()


def test_batch_external_big_entries_and_n40(lib):
    from permgpu.batch import batch_permanents
    rng = np.random.default_rng(5)
    mats = [rng.integers(-(1 << 45), 1 << 45, (5, 5), dtype=np.int64),
            rng.integers(-2, 3, (10, 10), dtype=np.int64)]
    got = batch_permanents(mats, tune=None)
    assert got == [oracle.exact_permanent(m.tolist()) for m in mats]


def test_autotune_persists_choice(lib, tmp_path):
    from permgpu import autotune, workloads
    mats = workloads.batch4096(count=64, seed=3)
    cache = tmp_path / "tune.json"
    best = autotune.tuned_parameters(mats, cache_path=str(cache),
                                     candidates=((12, 6, 2), (13, 6, 2)))
    assert cache.exists()
    assert autotune.tuned_parameters(mats, cache_path=str(cache)) == best
