"""GPU checks of the FP64 Glynn forward + hand-written gradient.

Tolerances are relative to the sum of |terms| each result is accumulated
from (returned by the kernel): 1e-10 for the forward and the gradient, the
bound the differentiable-permanent workload states.
"""

import json

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _t(a):
    import torch
    return torch.as_tensor(np.asarray(a, dtype=np.float64)).cuda()


def test_forward_matches_reference_float_code(lib):
    from permgpu.f64 import permanent_f64
    for c in json.loads((GOLDEN / "float_small.json").read_text())["cases"]:
        a = np.array(c["matrix"])
        if a.shape[0] < 2:
            continue
        per, _, s, _ = permanent_f64(_t(a)[None], want_grad=False)
        assert abs(per.item() - c["permanent"]) <= TOL * s.item()


@pytest.mark.parametrize("n", [2, 3, 4, 5, 8, 11, 13, 16, 17, 20])
def test_forward_and_gradient_vs_oracle(lib, n):
    from permgpu.f64 import permanent_f64
    rng = np.random.default_rng(700 + n)
    A = rng.normal(0, 1 / np.sqrt(n), (3, n, n))
    per, grad, s, gs = permanent_f64(_t(A))
    for b in range(3):
        want, _ = oracle.glynn_f64(A[b], 8)
        assert abs(per[b].item() - want) <= TOL * s[b].item()
        if n <= 13:
            g = oracle.glynn_f64_grad(A[b], 8)
            err = np.abs(grad[b].cpu().numpy() - g)
            assert (err <= TOL * gs[b].cpu().numpy()[:, None]).all()


def test_integer_valued_20x20_against_exact_minors(lib):
    from permgpu.f64 import permanent_f64
    data = json.loads((GOLDEN / "float20int_minors.json").read_text())
    for c in data["cases"]:
        A = np.array(c["matrix"], dtype=np.float64)
        per, grad, s, gs = permanent_f64(_t(A)[None])
        assert abs(per.item() - int(c["permanent"])) <= TOL * s.item()
        want = np.array([[float(int(x)) for x in row] for row in c["minors"]])
        err = np.abs(grad[0].cpu().numpy() - want)
        assert (err <= TOL * gs[0].cpu().numpy()[:, None]).all()


def test_row_expansion_identity_n28(lib):
    # size-independent property at the benchmark size: for every row i,
    # sum_j a_ij * d per / d a_ij = per(A)
    from permgpu import workloads
    from permgpu.f64 import permanent_f64
    A = workloads.float28(count=2)
    per, grad, s, gs = permanent_f64(_t(A))
    g = grad.cpu().numpy()
    for b in range(2):
        want, _ = oracle.glynn_f64(A[b], 16)
        assert abs(per[b].item() - want) <= TOL * s[b].item()
        expansion = (A[b] * g[b]).sum(axis=1)
        scale = (np.abs(A[b]) * gs[b].cpu().numpy()[:, None]).sum(axis=1)
        assert (np.abs(expansion - per[b].item()) <= 1e-9 * scale).all()


def test_central_finite_differences(lib):
    from permgpu.f64 import permanent_f64
    rng = np.random.default_rng(5)
    n, h = 10, 1e-6
    A = rng.normal(0, 1 / np.sqrt(n), (n, n))
    _, grad, _, _ = permanent_f64(_t(A)[None])
    for (i, j) in [(0, 0), (3, 7), (9, 2)]:
        Ap, Am = A.copy(), A.copy()
        Ap[i, j] += h
        Am[i, j] -= h
        fd = (oracle.glynn_f64(Ap, 4)[0] - oracle.glynn_f64(Am, 4)[0]) / (2 * h)
        assert abs(fd - grad[0, i, j].item()) <= 1e-6 * max(1.0, abs(fd))


def test_autograd_function(lib):
    import torch
    from permgpu.f64 import glynn_permanent
    rng = np.random.default_rng(8)
    A = _t(rng.normal(0, 0.3, (4, 7, 7))).requires_grad_(True)
    w = _t(rng.normal(0, 1, 4))
    loss = (glynn_permanent(A) * w).sum()
    loss.backward()
    for b in range(4):
        g = oracle.glynn_f64_grad(A[b].detach().cpu().numpy(), 2)
        assert np.allclose(A.grad[b].cpu().numpy(), w[b].item() * g, rtol=1e-10, atol=1e-12)
    # forward-only evaluation skips the gradient work and matches
    with torch.no_grad():
        per = glynn_permanent(A.detach())
    assert per.shape == (4,)


def test_complex_forward_matches_reference_and_oracle(lib):
    import torch
    from permgpu.f64 import permanent_c64, permanent_gpu
    for c in json.loads((GOLDEN / "float_small.json").read_text())["complex_cases"]:
        a = np.array(c["re"]) + 1j * np.array(c["im"])
        per, s = permanent_c64(torch.as_tensor(a).cuda()[None])
        assert abs(per.item() - complex(*c["permanent"])) <= TOL * s.item()
        assert abs(permanent_gpu(a) - complex(*c["permanent"])) <= TOL * s.item()
    rng = np.random.default_rng(41)
    for n in (13, 20):
        a = rng.normal(0, 0.2, (n, n)) + 1j * rng.normal(0, 0.2, (n, n))
        per, s = permanent_c64(torch.as_tensor(a).cuda()[None])
        want, ws = oracle.glynn_c64(a)
        assert abs(per.item() - want) <= TOL * s.item()
        assert abs(s.item() - ws) <= 1e-5 * ws


def test_small_orders_and_shapes(lib):
    import torch
    from permgpu.f64 import permanent_f64, permanent_float, permanent_gpu
    per, grad, _, _ = permanent_f64(torch.zeros(2, 0, 0, dtype=torch.float64, device="cuda"))
    assert per.tolist() == [1.0, 1.0]
    per, grad, _, _ = permanent_f64(_t([[[2.5]]]))
    assert per.item() == 2.5 and grad.item() == 1.0
    assert permanent_float([[1.0, 2.0], [3.0, 4.0]]) == 10.0
    assert permanent_gpu(np.zeros((0, 0))) == 1.0


def test_integer_valued_28x28_gradient_against_exact_minors(lib):
    # The workload's order with an exact oracle: integer-valued 28 x 28
    # matrices (entries in [-2, 2]); per(A) and all 784 minors
    # per(A without row i, column j) exactly from the exact engine (pinned
    # to the reference's perm.matrix_permanent), every FP64 gradient entry
    # within 1e-10 of its row's sum of |terms|
    from permgpu.f64 import permanent_f64
    rng = np.random.default_rng(55)
    n = 28
    for _ in range(2):
        A = rng.integers(-2, 3, (n, n)).astype(np.int64)
        minors = [np.delete(np.delete(A, i, 0), j, 1) for i in range(n) for j in range(n)]
        exact = np.array([float(v) for v in lib.batch_exact(minors)]).reshape(n, n)
        per, grad, s, gs = permanent_f64(_t(A)[None])
        assert abs(per.item() - lib.exact_permanent(A, lib.exact_limbs(A))) <= TOL * s.item()
        err = np.abs(grad[0].cpu().numpy() - exact)
        assert (err <= TOL * gs[0].cpu().numpy()[:, None]).all(), err.max()


def test_central_differences_n28(lib):
    # per is linear in each entry, so (per(A + h e_ij) - per(A - h e_ij)) / 2h
    # equals d per / d a_ij up to the forward's rounding (h = 1e-6): 16
    # entries of an N(0, 1/28) matrix, the 32 shifted matrices in one batch
    import torch
    from permgpu import workloads
    from permgpu.f64 import permanent_f64
    A = workloads.float28(count=1, seed=5)[0]
    n, h = 28, 1e-6
    _, grad, _, gs = permanent_f64(_t(A)[None])
    rng = np.random.default_rng(16)
    idx = [(int(i), int(j)) for i, j in zip(rng.integers(0, n, 16), rng.integers(0, n, 16))]
    shifted = []
    for i, j in idx:
        for sgn in (1, -1):
            B = A.copy()
            B[i, j] += sgn * h
            shifted.append(B)
    per, _, s, _ = permanent_f64(_t(np.stack(shifted)), want_grad=False)
    per, s = per.cpu().numpy(), s.cpu().numpy()
    for k, (i, j) in enumerate(idx):
        fd = (per[2 * k] - per[2 * k + 1]) / (2 * h)
        # rounding of the two forwards (measured near 1e-13 of their |terms|
        # sums; 1e-11 allowed) over 2h, plus the gradient's own tolerance
        bound = 1e-11 * (s[2 * k] + s[2 * k + 1]) / (2 * h) + TOL * gs[0, i].item()
        assert abs(fd - grad[0, i, j].item()) <= bound, (i, j)


def test_double_float_stress_cases(lib):
    # What FP32 pairs are weak at, against exact integer permanents:
    # rows scaled by 2^+-200 (FP32 alone overflows), near-equal rows whose
    # Glynn terms cancel deeply (1024 J + E), and a matrix whose permanent
    # is exactly 0 while its terms are large (block triangular with a
    # zero-permanent 2 x 2 block)
    from permgpu.f64 import permanent_f64
    rng = np.random.default_rng(77)
    n = 24
    A = rng.integers(-8, 9, (n, n)).astype(np.int64)
    exact = lib.exact_permanent(A, lib.exact_limbs(A))
    D = np.where(np.arange(n) % 2 == 0, 2.0 ** 200, 2.0 ** -200)
    per, _, s, _ = permanent_f64(_t(A * D[:, None])[None], want_grad=False)
    assert abs(per.item() - exact) <= TOL * s.item()
    base, _, sb, _ = permanent_f64(_t(A)[None], want_grad=False)
    assert per.item() == base.item() and s.item() == sb.item()   # power-of-two rows: bitwise

    C = 1024 + rng.integers(-1, 2, (n, n)).astype(np.int64)
    exact = lib.exact_permanent(C, lib.exact_limbs(C))
    per, _, s, _ = permanent_f64(_t(C)[None], want_grad=False)
    assert abs(per.item() - exact) <= TOL * s.item()
    assert abs(exact) < 1e-3 * s.item()          # the terms do cancel deeply

    Z = rng.integers(-8, 9, (n, n)).astype(np.int64)
    Z[:2, :2] = [[1, 1], [1, -1]]
    Z[2:, :2] = 0
    assert lib.exact_permanent(Z, lib.exact_limbs(Z)) == 0
    per, grad, s, gs = permanent_f64(_t(Z)[None])
    assert abs(per.item()) <= TOL * s.item()
    minors = [np.delete(np.delete(Z, i, 0), j, 1) for i in range(n) for j in range(n)]
    want = np.array([float(v) for v in lib.batch_exact(minors)]).reshape(n, n)
    assert (np.abs(grad[0].cpu().numpy() - want) <= TOL * gs[0].cpu().numpy()[:, None]).all()


@pytest.mark.parametrize("n", [2, 5, 10, 17, 21])
def test_window_kernel_whole_walks_vs_oracle(lib, n):
    # the window kernel (two rows per lane above 32) over the whole walk at
    # small orders, real and complex, against the CPU FP64 restatement
    from permgpu.f64 import glynn_window
    rng = np.random.default_rng(900 + n)
    A = rng.normal(0, 1 / np.sqrt(n), (n, n))
    got, s = glynn_window(A, 0, 1 << (n - 1))
    want, _ = oracle.glynn_f64(A, 8)
    assert abs(got / 2 ** (n - 1) - want) <= TOL * s / 2 ** (n - 1)
    C = A + 1j * rng.normal(0, 1 / np.sqrt(n), (n, n))
    got, s = glynn_window(C, 0, 1 << (n - 1))
    want, _ = oracle.glynn_c64(C)
    assert abs(got / 2 ** (n - 1) - want) <= TOL * s / 2 ** (n - 1)


def test_orders_above_32_whole_forward(lib):
    # permanent_parallel_real / _complex accept n <= 63
    # (perm_parallel_cuda.cu:358): a full 2^33-state forward at n = 34 of an
    # integer-valued matrix against the exact engine, and a complex n = 33
    # matrix D A (rows multiplied by 1, i, -1, -i: exact in floating point)
    # against prod(d) per(A)
    import torch
    from permgpu.f64 import permanent_c64, permanent_f64, permanent_gpu
    rng = np.random.default_rng(34)
    A = rng.integers(-2, 3, (34, 34)).astype(np.int64)
    exact = lib.exact_permanent(A, lib.exact_limbs(A))
    per, _, s, _ = permanent_f64(_t(A)[None], want_grad=False)
    assert abs(per.item() - exact) <= TOL * s.item()
    assert abs(permanent_gpu(A.astype(float)) - exact) <= TOL * s.item()
    B = rng.integers(-2, 3, (33, 33)).astype(np.int64)
    exact = lib.exact_permanent(B, lib.exact_limbs(B))
    d = np.array([1, 1j, -1, -1j])[rng.integers(0, 4, 33)]
    per, s = permanent_c64(torch.as_tensor(d[:, None] * B.astype(complex)).cuda()[None])
    assert abs(per.item() - np.prod(d) * exact) <= TOL * s.item()
    with pytest.raises(ValueError):
        permanent_f64(_t(A)[None])                 # the gradient stops at 32
    with pytest.raises(lib.PermGpuError):
        permanent_f64(_t(np.ones((64, 64)))[None], want_grad=False)


@pytest.mark.parametrize("n", [40, 48, 63])
def test_windows_at_large_orders(lib, n):
    # whole walks at these orders take minutes to centuries; windows of
    # 2^22 states at the start, the middle and the end against the exact
    # engine's unscaled window sums (n <= 48) or against the real window
    # times prod(d) for the complex D A (n = 63, no exact engine there)
    from permgpu import shard
    from permgpu.f64 import glynn_window
    rng = np.random.default_rng(1000 + n)
    A = rng.integers(-2, 3, (n, n)).astype(np.int64)
    d = np.array([1, 1j, -1, -1j])[rng.integers(0, 4, n)]
    states, w = 1 << (n - 1), 1 << 22
    for lo in (0, states // 2 + (1 << 24), states - w):
        got, s = glynn_window(A.astype(float), lo, lo + w)
        if n <= 48:
            want = float(shard.words_value(shard.exact_partial_words(A, lo, lo + w)))
            assert abs(got - want) <= TOL * s, (n, lo)
        gc, sc = glynn_window(d[:, None] * A.astype(complex), lo, lo + w)
        assert abs(gc - np.prod(d) * got) <= TOL * (s + sc), (n, lo)
    # dense real rows at n = 63: terms near 2^-200 stay representable
    G = rng.normal(0, 1 / np.sqrt(n), (n, n))
    got, s = glynn_window(G, 0, w)
    assert s > 0 and np.isfinite(got)
