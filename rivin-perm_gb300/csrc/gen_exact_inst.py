#!/usr/bin/env python3
"""Writes exact_inst_*.cu and exact_dispatch.cu: the compiled (order N,
group size G) shapes of the exact Glynn kernel (exact_glynn.cuh).

Group sizes: 1..4 for small orders; 5 and 6 from order 24; 7, 8 and 10
from order 24 for matrices with small row bounds (0/1 and sparse matrices:
a row of weight w allows about 31 / log2(w) rows per 32-bit group, and
fewer groups mean fewer multi-word products per term).  The shapes are
spread over PARTS translation units so that they compile in parallel.

    python gen_exact_inst.py      # run from any directory
"""

from pathlib import Path

HERE = Path(__file__).resolve().parent
PARTS = 12
MAX_G = 10


def shapes():
    out = []
    for n in range(2, 49):
        if n <= 3:
            gs = {n, 1} | ({2} if n == 3 else set())
        else:
            gs = {3, 4}
            if n >= 24:
                gs |= {5, 6, 7, 8, 10}
            if n <= 32:
                gs |= {2}
            if n <= 16:
                gs |= {1}
        out += [(n, g) for g in sorted(gs) if g <= n]
    return out


def key(n, g):
    return n * 16 + g


def main():
    sh = shapes()
    for f in HERE.glob("exact_inst_*.cu"):
        f.unlink()
    parts = [sh[i::PARTS] for i in range(PARTS)]
    for i, part in enumerate(parts):
        cases = "\n".join(
            f"    case {key(n, g)}:\n"
            f"        if (args) *err = launch_exact_glynn<{n}, {g}>(*args, blocks, stream);\n"
            f"        if (occ) *occ = occupancy_exact_glynn<{n}, {g}>();\n"
            f"        return true;" for n, g in part)
        (HERE / f"exact_inst_{i}.cu").write_text(
            f"// Instantiations of the exact Glynn kernel (part {i} of {PARTS}),\n"
            f"// written by gen_exact_inst.py.\n"
            f'#include "exact_glynn.cuh"\n\n'
            f"namespace pg {{\n\n"
            f"bool exact_dispatch_{i}(int N, int G, const ExactArgs *args, int blocks,\n"
            f"                       cudaStream_t stream, cudaError_t *err, int *occ) {{\n"
            f"    switch (N * 16 + G) {{\n{cases}\n"
            f"    default:\n        return false;\n    }}\n}}\n\n"
            f"}}  // namespace pg\n")
    decls = "\n".join(
        f"bool exact_dispatch_{i}(int, int, const ExactArgs *, int, cudaStream_t, "
        f"cudaError_t *, int *);" for i in range(PARTS))
    tries = "\n".join(
        f"    if (exact_dispatch_{i}(N, G, args, blocks, stream, err, occ)) return true;"
        for i in range(PARTS))
    cases = "\n".join(f"    case {key(n, g)}:" for n, g in sh)
    (HERE / "exact_dispatch.cu").write_text(f"""// Dispatch over the compiled (order, group size) pairs of the exact kernel,
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {{

{decls}

static bool dispatch(int N, int G, const ExactArgs *args, int blocks,
                     cudaStream_t stream, cudaError_t *err, int *occ) {{
{tries}
    return false;
}}

bool exact_compiled(int N, int G) {{
    if (N < 2 || N > 48 || G < 1 || G > EXACT_MAX_G) return false;
    switch (N * 16 + G) {{
{cases}
        return true;
    default:
        return false;
    }}
}}

cudaError_t launch_exact_any(int N, int G, const ExactArgs &args, int blocks,
                             cudaStream_t stream) {{
    cudaError_t err = cudaErrorInvalidValue;
    if (!dispatch(N, G, &args, blocks, stream, &err, nullptr)) return cudaErrorInvalidValue;
    return err;
}}

int occupancy_exact_any(int N, int G) {{
    cudaError_t err = cudaSuccess;
    int occ = 1;
    if (!dispatch(N, G, nullptr, 0, nullptr, &err, &occ)) return 1;
    return occ;
}}

}}  // namespace pg
""")
    print(f"{len(sh)} shapes in {PARTS} parts")


if __name__ == "__main__":
    main()
