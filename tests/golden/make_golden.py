"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout that has the reference (rivin-perm) at REFERENCE_DIR and
its OpenMP extensions built by oracle/build_ref.sh:

    oracle/build_ref.sh REFERENCE_DIR
    python tests/golden/make_golden.py --reference REFERENCE_DIR [--slow]

Every value is produced by the reference's own code: perm_c_ext /
perm_binary_ext (compiled from perm_c_omp.c / perm_binary_omp.c) and the
Python API (perm.matrix_permanent, perm.permanent, perm_binary.*).  The
published tables that the reference ships (schur_permanents.txt) and the
constants its tests pin (tests/test_cuda_device_schur_glynn.py:141-146,
tests/test_cuda_device_binary.py:30, BINARY_APPLICATIONS.md:157-160) are
recorded with their source.  --slow adds the 32x32 exact permanent and the
20x20 gradient-by-minors fixture (minutes of CPU time).
"""

from __future__ import annotations

import argparse
import json
import random
import re
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
INT64_MIN, INT64_MAX = -(1 << 63), (1 << 63) - 1


def dump(name, obj):
    (HERE / name).write_text(json.dumps(obj, indent=1, sort_keys=True) + "\n")
    print("wrote", name)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="the rivin-perm checkout the fixtures are generated from")
    ap.add_argument("--slow", action="store_true")
    ap.add_argument("--necklace-only", action="store_true",
                    help="regenerate only necklace_stats.json")
    ap.add_argument("--poly-only", action="store_true",
                    help="regenerate only poly.json")
    args = ap.parse_args()

    ref = Path(args.reference)
    sys.path.insert(0, str(REPO / "oracle" / "_ref"))
    sys.path.insert(0, str(ref))
    sys.path.insert(0, str(REPO / "rivin-perm_gb300"))
    import numpy as np
    import perm
    import perm_binary
    import perm_c_ext
    import perm_binary_ext
    from perm_binary_applications import grid_biadjacency
    from permgpu import workloads

    assert perm.HAS_C_EXT and perm_binary.HAS_BINARY_EXT

    # ---- necklace quotient statistics (tests/test_schur_cpu_glynn.py:120-130
    #      checks the same counts against Burnside's lemma) -------------------
    # ---- polynomial permanents (perm_polynomial.py, native engine built by
    #      oracle/build_ref.sh) ------------------------------------------
    if not args.necklace_only:
        import perm_polynomial as pp
        assert pp.polynomial_backend_capabilities()["native_extension_available"]
        prng = random.Random(20261203)
        affine, principal, rook, wrook = [], [], [], []
        for n in (0, 1, 2, 3, 5, 8, 11, 14, 16):
            c = [[prng.randint(-9, 9) for _ in range(n)] for _ in range(n)]
            l = [[prng.randint(-9, 9) for _ in range(n)] for _ in range(n)]
            mods = [3, 9, 1_000_003, 2_147_483_647, 3_037_000_501, INT64_MAX]
            affine.append({"constant": c, "linear": l,
                           "exact": [str(v) for v in pp.affine_permanent(c, l)],
                           "bounds": [str(v) for v in pp.affine_permanent_bounds(c, l)],
                           "moduli": mods,
                           "residues": [list(pp.affine_permanent_mod(c, l, m)) for m in mods]})
        big = [[prng.randint(-(1 << 50), 1 << 50) for _ in range(6)] for _ in range(6)]
        lin = [[prng.randint(0, 3) for _ in range(6)] for _ in range(6)]
        affine.append({"constant": big, "linear": lin,
                       "exact": [str(v) for v in pp.affine_permanent(big, lin)],
                       "bounds": [str(v) for v in pp.affine_permanent_bounds(big, lin)],
                       "moduli": [], "residues": []})
        for n in (4, 9, 13, 18):
            a = [[prng.randint(-4, 4) for _ in range(n)] for _ in range(n)]
            principal.append({"matrix": a,
                              "exact": [str(v) for v in pp.principal_permanent_polynomial(a)],
                              "mod_1000003": list(pp.principal_permanent_polynomial_mod(a, 1_000_003))})
        for n, dens in ((5, 0.5), (10, 0.4), (16, 0.5), (20, 0.3), (22, 0.5)):
            a = [[int(prng.random() < dens) for _ in range(n)] for _ in range(n)]
            rook.append({"matrix": a, "rook": [str(v) for v in pp.rook_polynomial(a)]})
        for n in (4, 8, 12, 15):
            a = [[prng.randint(0, 7) * (prng.random() < 0.6) for _ in range(n)] for _ in range(n)]
            wrook.append({"matrix": a, "rook": [str(v) for v in pp.weighted_rook_polynomial(a)]})
        dump("poly.json", {"source": "perm_polynomial (native engine perm_polynomial_omp.c)",
                           "affine": affine, "principal": principal, "rook": rook,
                           "weighted_rook": wrook})
        # ---- permanents mod 3 (perm_mod3.permanent_mod3_fast, OpenMP ext)
        import perm_mod3
        assert perm_mod3.HAS_MOD3_OMP
        mrng = np.random.default_rng(20261204)
        mod3 = []
        for n in (2, 3, 4, 7, 12, 17, 21, 26, 30, 32, 33):
            for low, high in ((-100, 100), (0, 2)):
                a = mrng.integers(low, high, (n, n)).astype(np.int64)
                mod3.append({"matrix": a.tolist(), "mod3": perm_mod3.permanent_mod3_fast(a)})
        dump("mod3.json", {"source": "perm_mod3.permanent_mod3_fast (perm_mod3_omp.c)",
                           "cases": mod3})
    if args.poly_only:
        return

    stats = {}
    for n in (3, 5, 7, 11, 13, 17, 19, 23, 29, 31):
        reps, words = perm_c_ext.schur_necklace_orbit_stats(n)
        stats[str(n)] = [reps, words]
    dump("necklace_stats.json", {"source": "perm_c_ext.schur_necklace_orbit_stats(n)",
                                 "stats": stats})
    if args.necklace_only:
        return

    # ---- generic residues across modulus tiers (tests/test_generic_native.py
    #      uses the same tiers and random.Random seeds) ----------------------
    cases = []
    moduli_tiers = [1, 2, 3, 6, 9, 15, 101, 2_147_483_647, 3_037_000_499,
                    3_037_000_501, INT64_MAX - 1, INT64_MAX]
    rng = random.Random(20260904)
    for order in range(7):
        for _ in range(3):
            m = [[rng.randrange(INT64_MIN, INT64_MAX + 1) for _ in range(order)]
                 for _ in range(order)]
            cases.append({"matrix": [[str(x) for x in r] for r in m], "moduli": moduli_tiers,
                          "residues": [perm_c_ext.permanent_mod_p(m, p, 1) for p in moduli_tiers]})
    rng = random.Random(161803)
    for modulus in (9, 25, 45):
        values = [-1, 0, 1] + [v for v in range(2, modulus) if modulus % v == 0]
        for order in (3, 5, 6):
            m = [[rng.choice(values) for _ in range(order)] for _ in range(order)]
            cases.append({"matrix": [[str(x) for x in r] for r in m], "moduli": [modulus],
                          "residues": [perm_c_ext.permanent_mod_p(m, modulus, 1)]})
    for order, modulus in ((16, 9), (17, 101), (18, 2_147_483_647), (18, INT64_MAX),
                           (20, 1_000_003), (21, 2_147_483_629)):
        rng = random.Random(271828 + order)
        m = [[rng.randrange(-modulus, modulus) for _ in range(order)] for _ in range(order)]
        cases.append({"matrix": [[str(x) for x in r] for r in m], "moduli": [modulus],
                      "residues": [perm_c_ext.permanent_mod_p(m, modulus, 8)]})
    dump("generic_residues.json", {"source": "perm_c_ext.permanent_mod_p (perm_c_omp.c)",
                                   "cases": cases})

    # ---- exact integer permanents via perm.matrix_permanent ---------------
    exact = []
    for n, seed, lo, hi in ((4, 1, -8, 8), (8, 2, -8, 8), (12, 3, -8, 8), (16, 4, -8, 8),
                            (20, 5, -8, 8), (22, 6, -3, 3), (13, 7, -3, 3), (27, 8, -3, 3),
                            (17, 9, -100, 100), (18, 10, -(1 << 20), 1 << 20)):
        a = workloads.generic_matrix(n, seed, lo, hi)
        t = time.time()
        v = perm.matrix_permanent(a.tolist(), method="generic")
        exact.append({"n": n, "seed": seed, "low": lo, "high": hi, "permanent": str(v),
                      "cpu_seconds": round(time.time() - t, 3)})
    a = workloads.generic24()
    t = time.time()
    v = perm.matrix_permanent(a.tolist(), method="generic")
    exact.append({"n": 24, "seed": 0, "low": -8, "high": 8, "permanent": str(v),
                  "cpu_seconds": round(time.time() - t, 3), "workload": "generic24"})
    dump("exact_generic.json", {"source": "perm.matrix_permanent(A, method='generic')",
                                "generator": "permgpu.workloads.generic_matrix(n, seed, low, high)",
                                "cases": exact})

    # ---- Schur ----------------------------------------------------------
    table = {}
    for line in (ref / "schur_permanents.txt").read_text().splitlines():
        mm = re.match(r"n=(\d+):\s+(-?\d+)", line.strip())
        if mm:
            table[int(mm.group(1))] = mm.group(2)
    schur_res = []
    for n in (3, 5, 7, 9, 11, 13, 15, 17, 19, 21, 23):
        for p in perm.find_primes_congruent_to_1_mod_n(n, 2, 1 << 30):
            w = perm.nth_root_of_unity_mod_p(n, p)
            schur_res.append({"n": n, "p": p, "omega": w,
                              "residue": perm_c_ext.schur_permanent_mod_p(n, w, p, 8)})
    # non-Glynn preconditions (full-matrix Ryser branch of perm_c_omp.c:1027-1047)
    for n, w, p in ((3, 1, 2), (3, 2, 5), (5, 3, 12), (4, 7, 101), (7, 5, 101)):
        schur_res.append({"n": n, "p": p, "omega": w,
                          "residue": perm_c_ext.schur_permanent_mod_p(n, w, p, 1)})
    exact_small = {n: str(perm.permanent(n)) for n in (3, 5, 7, 9, 11, 13, 15, 17, 19)}
    dump("schur.json", {
        "table_source": "schur_permanents.txt (OEIS A003112 + reference computations)",
        "table": table,
        "computed": exact_small,
        "residues": schur_res,
        "pins": [{"n": 33, "p": 4294967161, "omega": 2662262, "residue": 1428739342,
                  "source": "tests/test_cuda_device_schur_glynn.py:141-146"},
                 {"n": 41, "p": 4294966153, "omega": 782766686, "residue": 3889040436,
                  "source": "tests/test_cuda_device_schur_glynn.py:153-160"},
                 {"n": 47, "p": 4294967161, "omega": 1002938914, "residue": 4173217525,
                  "source": "tests/test_cuda_device_schur_glynn.py:163-172"}],
        "graham_lehmer": {str(n): list(perm._graham_lehmer_schur_congruence(n) or ())
                          for n in range(3, 48, 2)},
        "cpu_plan_prime_counts": {str(n): len(perm._plan_schur_exact_crt(
            n, 2 * perm.schur_permanent_bound(n) + 1, max(n + 1, 1 << 30))[0])
            for n in (31, 33)},
    })

    # ---- binary -----------------------------------------------------------
    grid = grid_biadjacency((4, 4, 5), periodic_axes=(0, 1))
    bin_cases = []
    rng = np.random.default_rng(20260815)
    for order in (2, 3, 5, 7, 8, 12, 16, 20):
        m = rng.integers(0, 2, (order, order)).astype(int).tolist()
        bin_cases.append({"matrix": m, "permanent": str(perm_binary.binary_permanent(m)),
                          "residues": {str(p): perm_binary_ext.binary_permanent_mod_p(m, p, 1)
                                       for p in (101, 2_147_483_647)}})
    m = [[1] * 13 for _ in range(13)]
    bin_cases.append({"matrix": m, "permanent": str(perm_binary.binary_permanent(m))})
    dense = []
    for i, mat in enumerate(workloads.binary40(8)):
        feasible, blocks = perm_binary._matching_blocks(perm_binary._row_masks(mat.tolist()))
        sizes = sorted(len(b) for b in blocks)
        bounds = [perm_binary._normalized_bound(perm_binary._unpack_masks(b)).bit_length()
                  for b in blocks if len(b) > 1]
        dense.append({"seed": 300 + i, "feasible": feasible, "block_sizes": sizes,
                      "bound_bits": bounds})
    mid = []
    for n, seed in ((24, 1), (26, 2), (28, 3)):
        mat = (np.random.default_rng(seed).random((n, n)) < 0.5).astype(int).tolist()
        t = time.time()
        r = perm_binary_ext.binary_permanent_mod_p(mat, 2_147_483_647, 8)
        mid.append({"n": n, "seed": seed, "p": 2_147_483_647, "residue": r,
                    "cpu_seconds": round(time.time() - t, 3)})
    dump("binary.json", {
        "grid_4x4x5_periodic01": {"matrix": grid, "permanent": "2551276235535120",
                                  "source": "tests/test_cuda_device_binary.py:30",
                                  "residues": {"2147483647": 1238389710, "2147483629": 1259774250},
                                  "residues_source": "BINARY_APPLICATIONS.md:157-160",
                                  "reference_crt_primes": list(perm_binary._crt_primes_above_bound(
                                      perm_binary.binary_permanent_bound(grid)))},
        "cases": bin_cases,
        "binary40_preprocessing": dense,
        "bernoulli_residues": mid,
        "generator": "bernoulli: (default_rng(seed).random((n,n)) < 0.5)",
    })

    # ---- floating point (reference CPU float code) -----------------------
    import perm_float
    fl = []
    rng = np.random.default_rng(77)
    for n in (2, 3, 5, 8, 10, 12):
        a = rng.normal(0, 1 / np.sqrt(n), (n, n))
        fl.append({"matrix": a.tolist(), "permanent": float(perm_float.permanent_float(a))})
    cx = []
    for n in (2, 3, 5, 8, 10):
        a = rng.normal(0, 1 / np.sqrt(2 * n), (n, n)) + 1j * rng.normal(0, 1 / np.sqrt(2 * n), (n, n))
        v = complex(perm_float.permanent_float(a))
        cx.append({"re": a.real.tolist(), "im": a.imag.tolist(), "permanent": [v.real, v.imag]})
    dump("float_small.json", {"source": "perm_float.permanent_float (Ryser + Kahan)", "cases": fl,
                              "complex_cases": cx})

    if args.slow and not (HERE / "exact_generic32.json").exists():
        a = workloads.generic32()
        t = time.time()
        v = perm.matrix_permanent(a.tolist(), method="generic")
        dump("exact_generic32.json", {"n": 32, "seed": 32, "low": -8, "high": 8,
                                      "permanent": str(v), "workload": "generic32",
                                      "cpu_seconds": round(time.time() - t, 1),
                                      "source": "perm.matrix_permanent(A, method='generic')"})
    if args.slow:
        mats = workloads.float20int(2)
        out = []
        for a in mats:
            ai = a.astype(int).tolist()
            n = len(ai)
            per = perm.matrix_permanent(ai, method="generic")
            grad = [[str(perm.matrix_permanent([r[:j] + r[j + 1:] for k, r in enumerate(ai) if k != i],
                                               method="generic")) for j in range(n)] for i in range(n)]
            out.append({"matrix": ai, "permanent": str(per), "minors": grad})
        dump("float20int_minors.json", {"source": "perm.matrix_permanent on A and every minor",
                                        "generator": "permgpu.workloads.float20int(2)",
                                        "cases": out})


if __name__ == "__main__":
    main()
