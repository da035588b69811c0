"""GPU checks of the host-pointer convenience entry points: the FP64
forward+gradient (pg_glynn_f64_fwd_bwd) and per-matrix residue lists for a
batch (pg_batch_residues), against the oracle."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
TOL = 1e-10


def test_f64_host_entry_matches_oracle(lib):
    rng = np.random.default_rng(61)
    for n in (2, 5, 9, 12):
        a = rng.normal(0, 1 / np.sqrt(n), (3, n, n))
        per, grad, s = lib.glynn_f64_fwd_bwd(a)
        for b in range(3):
            want, _ = oracle.glynn_f64(a[b], 4)
            assert abs(per[b] - want) <= TOL * s[b]
            g = oracle.glynn_f64_grad(a[b], 4)
            assert np.allclose(grad[b], g, rtol=1e-9, atol=1e-12)
        per2, none, _ = lib.glynn_f64_fwd_bwd(a, want_grad=False)
        assert none is None and np.array_equal(per, per2)
    per, grad, s = lib.glynn_f64_fwd_bwd(np.array([[[2.5]], [[-1.0]]]))
    assert per.tolist() == [2.5, -1.0] and grad.ravel().tolist() == [1.0, 1.0]


def test_batch_residues_mixed_batch(lib):
    rng = np.random.default_rng(62)
    mats, mods = [], []
    for n in (0, 1, 2, 5, 9, 14, 17, 20):
        mats.append(rng.integers(-9, 10, (n, n)))
        mods.append([3, 101, 1_000_003, 2_147_483_647, (1 << 61) - 1, 6, 1 << 20][: 2 + n % 5])
    # entries too large for the exact engine take the residue path
    big = rng.integers(-(1 << 62), 1 << 62, (11, 11))
    mats.append(big)
    mods.append([1_000_003, 2_147_483_629, (1 << 62) + 135])
    got = lib.batch_residues(mats, mods)
    for m, ms, row in zip(mats, mods, got):
        assert row == [oracle.permanent_mod_p(m, q, 4) for q in ms], m.shape


def test_c64_host_entry_matches_oracle(lib):
    rng = np.random.default_rng(63)
    for n in (2, 6, 11, 14):
        a = (rng.normal(0, 1 / np.sqrt(n), (3, n, n))
             + 1j * rng.normal(0, 1 / np.sqrt(n), (3, n, n)))
        per, s = lib.glynn_c64(a)
        for b in range(3):
            want, _ = oracle.glynn_c64(a[b])
            assert abs(per[b] - want) <= TOL * s[b]
    per, s = lib.glynn_c64(np.array([[[2.5 - 1j]], [[-1.0 + 3j]]]))
    assert per.tolist() == [2.5 - 1j, -1.0 + 3j]
