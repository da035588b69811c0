"""Seeded synthetic workloads (numpy default_rng), shared by the tests, the
golden-fixture generator and bench.py.

  generic24   one 24x24 int64 matrix, entries U[-8,8], seed 0
  generic32   one 32x32 int64 matrix, entries U[-8,8], seed 32
  schur       perm(S_31), perm(S_33) (deterministic)
  binary40    eight 40x40 Bernoulli(0.5) 0/1 matrices, seeds 300..307
  batch4096   4096 int64 matrices, n ~ U[12,28], entries U[-3,3], seed 4
  float28     256 float64 matrices 28x28, entries N(0, 1/28), seed 5
  float20int  k integer-valued 20x20 float64 matrices, entries U[-2,2], seed 55
"""

from __future__ import annotations

from typing import List

import numpy as np


def generic_matrix(n: int, seed: int, low: int = -8, high: int = 8) -> np.ndarray:
    return np.random.default_rng(seed).integers(low, high + 1, (n, n), dtype=np.int64)


def generic24() -> np.ndarray:
    return generic_matrix(24, 0)


def generic32() -> np.ndarray:
    return generic_matrix(32, 32)


def binary40(count: int = 8, n: int = 40) -> List[np.ndarray]:
    return [(np.random.default_rng(300 + i).random((n, n)) < 0.5).astype(np.uint8)
            for i in range(count)]


def batch4096(count: int = 4096, seed: int = 4, n_lo: int = 12, n_hi: int = 28,
              low: int = -3, high: int = 3) -> List[np.ndarray]:
    rng = np.random.default_rng(seed)
    orders = rng.integers(n_lo, n_hi + 1, count)
    return [rng.integers(low, high + 1, (int(n), int(n)), dtype=np.int64) for n in orders]


def float28(count: int = 256, n: int = 28, seed: int = 5) -> np.ndarray:
    return np.random.default_rng(seed).normal(0.0, 1.0 / np.sqrt(n), (count, n, n))


def float20int(count: int = 2, n: int = 20, seed: int = 55) -> np.ndarray:
    return np.random.default_rng(seed).integers(-2, 3, (count, n, n)).astype(np.float64)
