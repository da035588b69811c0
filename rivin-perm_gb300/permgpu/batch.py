"""Batched exact permanents: thousands of integer matrices of uneven order
in one persistent, graph-captured GPU launch.

    batch_permanents(matrices, tune="auto") -> [per(A) for A in matrices]

The reference evaluates such a workload as a Python loop of
perm.matrix_permanent calls (perm.py:1076-1212, one prime at a time); here
every (matrix, Gray range) task of the whole batch is scheduled by one
work-stealing kernel.  Results are bit-exact with the per-matrix path.
Matrices outside the exact engine's range go through
permgpu.matrix_permanent individually (residues + CRT).
"""

from __future__ import annotations

from typing import List, Sequence

import numpy as np

from . import _lib
from .generic import matrix_permanent


def _exact_ok(m: np.ndarray) -> bool:
    n = m.shape[0] if m.ndim == 2 else 0
    if n <= 1:
        return True
    if np.abs(m).max(initial=0) >= (1 << 40):
        return False
    return _lib.exact_supported(m)


def batch_permanents(matrices: Sequence, tune="auto", cache_path=None) -> List[int]:
    """Exact permanents of a list of square integer matrices.

    ``tune``: "auto" (autotuned parameters from the persisted cache, tuning
    once if absent), None (library defaults) or a (lane_log_states,
    chunk_log_len, blocks_per_sm) tuple.
    """
    mats = [np.asarray(m, dtype=np.int64).reshape(len(m), len(m)) if len(m) else
            np.zeros((0, 0), np.int64) for m in matrices]
    ok = [i for i, m in enumerate(mats) if _exact_ok(m)]
    out: List[int] = [0] * len(mats)
    if ok:
        sub = [mats[i] for i in ok]
        if tune == "auto":
            from .autotune import tuned_parameters
            tune = tuned_parameters(sub, cache_path=cache_path)
        plan = _lib.BatchPlan(sub, tune)
        try:
            plan.launch()
            for i, v in zip(ok, plan.results()):
                out[i] = v
        finally:
            plan.close()
    in_batch = set(ok)
    for i, m in enumerate(mats):
        if i not in in_batch:
            out[i] = matrix_permanent(m.tolist())
    return out
