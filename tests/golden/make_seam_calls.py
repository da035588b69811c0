"""Record the calls rivin-perm's Python API makes through its native seams.

The reference's perm.py and perm_binary.py reach their compiled extensions
only through module attributes (perm.perm_c_ext: permanent_mod_p,
ryser_permanent_mod_p, schur_permanent_mod_p, get_max_threads;
perm_binary._binary_ext: binary_permanent_mod_p).  This script runs the
reference's own public API with a recording proxy around the real compiled
extensions (built by oracle/build_ref.sh into oracle/_ref) and writes every
call, its arguments and its result to seam_calls.json, together with the
API's final results.  tests/test_gpu_dropin.py replays the recorded calls
on permgpu.GpuExt / BinaryGpuExt: a drop-in that returns the recorded value
for every call gives the reference's API the same final result.

    oracle/build_ref.sh REFERENCE_DIR
    python tests/golden/make_seam_calls.py --reference REFERENCE_DIR
"""

from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]


class Recorder:
    """Forwards to the real extension and logs (method, args, result)."""

    def __init__(self, real, log, names):
        self._real, self._log, self._names = real, log, names

    def __getattr__(self, name):
        target = getattr(self._real, name)
        if name not in self._names or not callable(target):
            return target

        def call(*args):
            result = target(*args)
            self._log.append({"fn": name, "args": args, "result": result})
            return result
        return call


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="the rivin-perm checkout whose API is recorded")
    args = ap.parse_args()
    sys.path.insert(0, str(REPO / "oracle" / "_ref"))
    sys.path.insert(0, str(Path(args.reference)))
    import numpy as np
    import perm
    import perm_binary
    import perm_c_ext
    import perm_binary_ext

    log: list = []
    perm.perm_c_ext = Recorder(perm_c_ext, log, {"permanent_mod_p", "ryser_permanent_mod_p",
                                                 "schur_permanent_mod_p"})
    perm.HAS_C_EXT = True
    perm_binary._binary_ext = Recorder(perm_binary_ext, log, {"binary_permanent_mod_p"})
    perm_binary.HAS_BINARY_EXT = True

    cases = []
    rng = np.random.default_rng(4242)
    for n, lo, hi in ((9, -8, 8), (14, -3, 3), (18, -(1 << 20), 1 << 20)):
        a = rng.integers(lo, hi + 1, (n, n)).tolist()
        start = len(log)
        value = perm.matrix_permanent(a, method="generic", parallel=False)
        cases.append({"api": "perm.matrix_permanent", "matrix": a, "result": str(value),
                      "calls": log[start:]})
    for n in (13, 17, 19):
        start = len(log)
        value = perm.permanent(n, parallel=False)
        cases.append({"api": "perm.permanent", "n": n, "result": str(value),
                      "calls": log[start:]})
    for n, density in ((12, 0.5), (16, 0.35)):
        m = (rng.random((n, n)) < density).astype(int).tolist()
        start = len(log)
        value = perm_binary.binary_permanent(m)
        cases.append({"api": "perm_binary.binary_permanent", "matrix": m, "result": str(value),
                      "calls": log[start:]})
    for c in cases:
        for call in c["calls"]:
            call["args"] = [a if not isinstance(a, int) else a for a in call["args"]]
    (HERE / "seam_calls.json").write_text(json.dumps({
        "source": "rivin-perm perm.matrix_permanent / perm.permanent / "
                  "perm_binary.binary_permanent with recording proxies around the compiled "
                  "perm_c_ext and perm_binary_ext (perm.py:917-923, 752-753; "
                  "perm_binary.py:822-824)",
        "cases": cases}, indent=1) + "\n")
    print("wrote seam_calls.json:", sum(len(c["calls"]) for c in cases), "calls")


if __name__ == "__main__":
    main()
