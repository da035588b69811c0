#!/usr/bin/env python3
"""Writes col_acc.cuh: the inline-PTX signed multi-word products (MulWordS)
and the column folds (FoldCols) of the exact Glynn term, for up to 15 words.

    python gen_col_acc.py      # run from any directory
"""

from pathlib import Path

HERE = Path(__file__).resolve().parent
LMAX = 15
out = []
w = out.append
w("""// Column accumulation of exact Glynn terms.
//
// A term is (-1)^sign * prod_g |x_g| over the row-group products x_g.  The
// sign is folded into the first group, so the running product R of the
// leading groups is a signed multi-word integer (little-endian 32-bit
// words, the top word two's complement).  MulWordS multiplies it by the next
// group magnitude (0 <= y < 2^31): the lower words with mul.wide.u32, the top
// word with mul.wide.s32, one add.cc/addc chain over the halves.
//
// The last group is not multiplied into R: its magnitude y multiplies each
// word of R into a 64-bit column accumulator (mad.wide, no carries), and
// FoldCols adds the columns into the two's-complement term accumulator once
// every few terms.  The host bounds y so that the columns cannot overflow
// between folds (terms per fold * y <= 2^32).
#pragma once
#include <stdint.h>

namespace pg {

// R[0..L-1] (signed top word) *= y, giving R[0..L]; 0 <= y < 2^31.
template <int L>
struct MulWordS {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        uint32_t carry = 0;
#pragma unroll
        for (int l = 0; l < L - 1; l++) {
            const uint64_t t = (uint64_t)R[l] * y + carry;
            R[l] = (uint32_t)t;
            carry = (uint32_t)(t >> 32);
        }
        const int64_t t = (int64_t)(int32_t)R[L - 1] * (int64_t)y + carry;
        R[L - 1] = (uint32_t)t;
        R[L] = (uint32_t)((uint64_t)t >> 32);
    }
};
""")
for L in range(1, LMAX + 1):
    body = []
    body.append(".reg .u64 w;")
    body.append(f".reg .u32 lo<{L}>, hi<{L}>;")
    for l in range(L):
        ty = "s32" if l == L - 1 else "u32"
        body.append(f"mul.wide.{ty} w, %{l}, %{L+1};")
        body.append(f"mov.b64 {{lo{l}, hi{l}}}, w;")
    if L == 1:
        body.append("mov.b32 %0, lo0;")
        body.append("mov.b32 %1, hi0;")
    else:
        body.append("mov.b32 %0, lo0;")
        body.append("add.cc.u32 %1, lo1, hi0;")
        for l in range(2, L):
            body.append(f"addc.cc.u32 %{l}, lo{l}, hi{l-1};")
        body.append(f"addc.u32 %{L}, hi{L-1}, 0;")
    outs = ", ".join([f'"+r"(R[{l}])' for l in range(L)] + [f'"=r"(R[{L}])'])
    w(f"""template <>
struct MulWordS<{L}> {{
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {{
        asm("{{\\n\\t"
""" + "".join(f'            "{b}\\n\\t"\n' for b in body) + f"""            "}}"
            : {outs}
            : "r"(y));
    }}
}};
""")

w("""// acc[0..NL-1] (two's complement) += sum_{l < NR-1} col[l] * 2^(32 l)
//                                    + colt * 2^(32 (NR-1))   (colt signed)
// as two carry chains: the low halves at their own word, the high halves one
// word up, the sign of colt extended above.  Needs NL >= NR + 1.
template <int NR, int NL>
struct FoldCols {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        uint64_t carry = 0;
#pragma unroll
        for (int l = 0; l < NL; l++) {
            uint64_t t = (uint64_t)acc[l] + carry;
            if (l < NR - 1) t += (uint32_t)col[l];
            if (l == NR - 1) t += (uint32_t)(uint64_t)colt;
            if (l >= 1 && l - 1 < NR - 1) t += (uint32_t)(col[l - 1] >> 32);
            if (l == NR) t += (uint32_t)((uint64_t)colt >> 32);
            if (l > NR) t += (uint32_t)(colt >> 63);
            acc[l] = (uint32_t)t;
            carry = t >> 32;
        }
    }
};
""")

def fold_ptx(NR, NL):
    body = []
    # operands: acc 0..NL-1 ("+r"), col 0..NR-2 ("l"), colt ("l")
    ci = lambda l: NL + l
    ct = NL + NR - 1
    body.append(f".reg .u32 clo<{NR}>, chi<{NR}>, ext;")
    for l in range(NR - 1):
        body.append(f"mov.b64 {{clo{l}, chi{l}}}, %{ci(l)};")
    body.append(f"mov.b64 {{clo{NR-1}, chi{NR-1}}}, %{ct};")
    body.append(f"shr.s32 ext, chi{NR-1}, 31;")
    # pass 1: low halves
    for l in range(NL):
        src = f"clo{l}" if l < NR else "0"
        op = "add.cc.u32" if l == 0 else ("addc.u32" if l == NL - 1 else "addc.cc.u32")
        body.append(f"{op} %{l}, %{l}, {src};")
    # pass 2: high halves, one word up
    for l in range(1, NL):
        src = f"chi{l-1}" if l - 1 < NR else "ext"
        op = "add.cc.u32" if l == 1 else ("addc.u32" if l == NL - 1 else "addc.cc.u32")
        body.append(f"{op} %{l}, %{l}, {src};")
    outs = ", ".join(f'"+r"(acc[{l}])' for l in range(NL))
    ins = ", ".join([f'"l"(col[{l}])' for l in range(NR - 1)] + ['"l"(colt)'])
    return f"""template <>
struct FoldCols<{NR}, {NL}> {{
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {{
        asm("{{\\n\\t"
""" + "".join(f'            "{b}\\n\\t"\n' for b in body) + f"""            "}}"
            : {outs}
            : {ins});
    }}
}};
"""

for NR in range(1, LMAX + 1):
    for extra in (1, 2, 3):
        NL = NR + extra
        if NL > 16:
            continue
        if NR == 1:
            # col[] is empty: pass a dummy pointer use-free variant
            pass
        w(fold_ptx(NR, NL))

w("}  // namespace pg\n")


def main():
    (HERE / "col_acc.cuh").write_text("\n".join(out))


if __name__ == "__main__":
    main()
