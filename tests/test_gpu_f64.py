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
