"""Autotuner for the batched engine's launch parameters.

Searches (lane_log_states, chunk_log_len, blocks_per_sm) — the work per
lane per task, the aligned chunk length, and the resident blocks per SM —
by timing the graph-captured batch launch with CUDA events, and persists
the winner in a JSON cache keyed by GPU name and a signature of the batch
(histogram of matrix orders).  Later calls with a matching key reuse it.
"""

from __future__ import annotations

import hashlib
import json
import os
import time
from pathlib import Path
from typing import Iterable, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib

DEFAULT_CANDIDATES: Tuple[Tuple[int, int, int], ...] = (
    (13, 6, 2), (12, 6, 2), (14, 6, 2), (15, 6, 2),
    (13, 5, 2), (13, 8, 2), (13, 6, 1), (11, 5, 2),
)

Tune = Tuple[int, int, int]


def cache_file(path: Optional[str] = None) -> Path:
    if path:
        return Path(path)
    env = os.environ.get("PERMGPU_TUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "permgpu" / "batch_tune.json"


def signature(matrices: Sequence[np.ndarray]) -> str:
    orders = np.bincount([np.asarray(m).shape[0] for m in matrices], minlength=64)
    return hashlib.sha1(orders.tobytes()).hexdigest()[:16]


def gpu_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown-gpu"


def _time_plan(plan: "_lib.BatchPlan", reps: int) -> float:
    import torch
    stream = torch.cuda.Stream()
    ptr = stream.cuda_stream
    plan.launch(ptr)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.launch(ptr)
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def autotune(matrices: Sequence[np.ndarray], candidates: Iterable[Tune] = DEFAULT_CANDIDATES,
             reps: int = 3, check: bool = True) -> Tuple[Tune, List[Tuple[Tune, float]]]:
    """Time every candidate on this batch; returns (best, [(tune, ms)])."""
    results = []
    reference = None
    for cand in candidates:
        plan = _lib.BatchPlan(matrices, cand)
        try:
            ms = _time_plan(plan, reps)
            if check:
                vals = plan.results()
                if reference is None:
                    reference = vals
                elif vals != reference:
                    raise RuntimeError(f"tuning candidate {cand} changed the results")
        finally:
            plan.close()
        results.append((tuple(cand), ms))
    best = min(results, key=lambda r: r[1])[0]
    return best, results


def tuned_parameters(matrices: Sequence[np.ndarray], cache_path: Optional[str] = None,
                     candidates: Iterable[Tune] = DEFAULT_CANDIDATES) -> Tune:
    """Cached tuning result for this GPU and batch signature (tunes on miss)."""
    path = cache_file(cache_path)
    key = f"{gpu_name()}|{signature(matrices)}"
    data = {}
    if path.exists():
        try:
            data = json.loads(path.read_text())
        except (OSError, ValueError):
            data = {}
    if key in data:
        return tuple(data[key]["tune"])
    best, results = autotune(matrices, candidates)
    data[key] = {"tune": list(best), "timings_ms": [[list(t), ms] for t, ms in results],
                 "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(data, indent=1, sort_keys=True))
    except OSError:
        pass
    return best
