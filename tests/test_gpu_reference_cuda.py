"""Parity with the reference's own CUDA kernels, run on the same GPU.

oracle/build_ref.sh compiles the device code of the reference's CUDA tools
unmodified into cubins; oracle/ref_cuda.py launches them with the host logic
of perm_modp_cuda.cu, perm_binary_cuda.cu and perm_parallel_cuda.cu restated.
Every residue they return must equal this repository's (integers: zero
tolerance), and the reference's FP64 Glynn value must agree with the
double-float forward within 1e-12 of sum |terms|.  The cubins are built where
the reference checkout exists and travel with the tree; without them these
tests skip.
"""

import math

import numpy as np
import pytest

import ref_cuda

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cuda.available(), reason="reference cubins not built")]

P30 = 1073741827          # the reference planner's first prime above 2^30 (perm.py:1122-1127)


@pytest.mark.parametrize("n,p", [(6, P30), (13, P30), (19, P30), (21, P30),
                                 (9, 2_305_843_009_213_693_951), (14, 1_000_000_007)])
def test_ryser_kernel_residues(lib, n, p):
    a = np.random.default_rng(100 + n).integers(-8, 9, (n, n), dtype=np.int64)
    assert ref_cuda.permanent_modp(a, p) == lib.residues(a, [p])[0]


@pytest.mark.parametrize("n,p", [(5, 2_147_483_647), (17, P30), (22, 4_294_967_291)])
def test_generic_glynn_kernel_residues(lib, n, p):
    a = np.random.default_rng(200 + n).integers(-8, 9, (n, n), dtype=np.int64)
    assert ref_cuda.glynn_modp(a, p) == lib.residues(a, [p])[0]


@pytest.mark.parametrize("n,p", [(28, 4_294_967_291), (30, 4_294_967_279)])
def test_pseudo_mersenne_glynn_kernel_residues(lib, n, p):
    a = np.random.default_rng(300 + n).integers(-8, 9, (n, n), dtype=np.int64)
    assert ref_cuda.glynn_modp(a, p) == lib.residues(a, [p])[0]


@pytest.mark.parametrize("n,density", [(12, 0.5), (20, 0.4), (26, 0.5)])
def test_binary_ratio_kernel_residues(lib, n, density):
    p = 2_147_483_647
    m = (np.random.default_rng(400 + n).random((n, n)) < density).astype(np.int64)
    m[np.arange(n), np.arange(n)] = 1            # no empty row or column
    assert ref_cuda.binary_modp(m, p) == lib.binary_residues(m, [p])[0]
    assert ref_cuda.binary_modp(m, p) == lib.exact_permanent(m, lib.exact_limbs(m)) % p


def test_binary_ratio_kernel_zero_row(lib):
    m = np.ones((10, 10), dtype=np.int64)
    m[3] = 0
    assert ref_cuda.binary_modp(m, 2_147_483_647) == 0


@pytest.mark.parametrize("n", [8, 16, 21])
def test_fp64_glynn_kernel_values(lib, n):
    a = np.random.default_rng(500 + n).normal(0.0, 1.0 / math.sqrt(n), (n, n))
    ref = ref_cuda.parallel_real(a)
    per, _, abs_sum = lib.glynn_f64_fwd_bwd(a[None], want_grad=False)
    assert abs(ref - per[0]) <= 1e-12 * abs_sum[0]


def test_necklace_kernel_residue_s41(lib):
    # the reference's persistent necklace kernel (M = 40, prefix depth 24),
    # one of the three 2^32 - c primes its planner takes for perm(S_41);
    # about 6 s of GPU time
    from permgpu.crt import nth_root_of_unity
    primes, _ = ref_cuda.schur_gpu_primes(41)
    assert len(primes) == 3
    q = primes[0]
    w = nth_root_of_unity(41, q)
    assert ref_cuda.schur_necklace_modp(41, w, q) == lib.schur_residues(41, [q], [w])[0]
