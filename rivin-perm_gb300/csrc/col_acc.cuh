// Column accumulation of exact Glynn terms.
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

template <>
struct MulWordS<1> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<1>, hi<1>;\n\t"
            "mul.wide.s32 w, %0, %2;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "mov.b32 %1, hi0;\n\t"
            "}"
            : "+r"(R[0]), "=r"(R[1])
            : "r"(y));
    }
};

template <>
struct MulWordS<2> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<2>, hi<2>;\n\t"
            "mul.wide.u32 w, %0, %3;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.s32 w, %1, %3;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.u32 %2, hi1, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "=r"(R[2])
            : "r"(y));
    }
};

template <>
struct MulWordS<3> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<3>, hi<3>;\n\t"
            "mul.wide.u32 w, %0, %4;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %4;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.s32 w, %2, %4;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.u32 %3, hi2, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "=r"(R[3])
            : "r"(y));
    }
};

template <>
struct MulWordS<4> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<4>, hi<4>;\n\t"
            "mul.wide.u32 w, %0, %5;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %5;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %5;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.s32 w, %3, %5;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.u32 %4, hi3, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "=r"(R[4])
            : "r"(y));
    }
};

template <>
struct MulWordS<5> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<5>, hi<5>;\n\t"
            "mul.wide.u32 w, %0, %6;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %6;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %6;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %6;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.s32 w, %4, %6;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.u32 %5, hi4, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "=r"(R[5])
            : "r"(y));
    }
};

template <>
struct MulWordS<6> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<6>, hi<6>;\n\t"
            "mul.wide.u32 w, %0, %7;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %7;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %7;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %7;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %7;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.s32 w, %5, %7;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.u32 %6, hi5, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "=r"(R[6])
            : "r"(y));
    }
};

template <>
struct MulWordS<7> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<7>, hi<7>;\n\t"
            "mul.wide.u32 w, %0, %8;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %8;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %8;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %8;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %8;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.u32 w, %5, %8;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mul.wide.s32 w, %6, %8;\n\t"
            "mov.b64 {lo6, hi6}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.cc.u32 %6, lo6, hi5;\n\t"
            "addc.u32 %7, hi6, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "=r"(R[7])
            : "r"(y));
    }
};

template <>
struct MulWordS<8> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<8>, hi<8>;\n\t"
            "mul.wide.u32 w, %0, %9;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %9;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %9;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %9;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %9;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.u32 w, %5, %9;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mul.wide.u32 w, %6, %9;\n\t"
            "mov.b64 {lo6, hi6}, w;\n\t"
            "mul.wide.s32 w, %7, %9;\n\t"
            "mov.b64 {lo7, hi7}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.cc.u32 %6, lo6, hi5;\n\t"
            "addc.cc.u32 %7, lo7, hi6;\n\t"
            "addc.u32 %8, hi7, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "+r"(R[7]), "=r"(R[8])
            : "r"(y));
    }
};

template <>
struct MulWordS<9> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<9>, hi<9>;\n\t"
            "mul.wide.u32 w, %0, %10;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %10;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %10;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %10;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %10;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.u32 w, %5, %10;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mul.wide.u32 w, %6, %10;\n\t"
            "mov.b64 {lo6, hi6}, w;\n\t"
            "mul.wide.u32 w, %7, %10;\n\t"
            "mov.b64 {lo7, hi7}, w;\n\t"
            "mul.wide.s32 w, %8, %10;\n\t"
            "mov.b64 {lo8, hi8}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.cc.u32 %6, lo6, hi5;\n\t"
            "addc.cc.u32 %7, lo7, hi6;\n\t"
            "addc.cc.u32 %8, lo8, hi7;\n\t"
            "addc.u32 %9, hi8, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "+r"(R[7]), "+r"(R[8]), "=r"(R[9])
            : "r"(y));
    }
};

template <>
struct MulWordS<10> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<10>, hi<10>;\n\t"
            "mul.wide.u32 w, %0, %11;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %11;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %11;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %11;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %11;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.u32 w, %5, %11;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mul.wide.u32 w, %6, %11;\n\t"
            "mov.b64 {lo6, hi6}, w;\n\t"
            "mul.wide.u32 w, %7, %11;\n\t"
            "mov.b64 {lo7, hi7}, w;\n\t"
            "mul.wide.u32 w, %8, %11;\n\t"
            "mov.b64 {lo8, hi8}, w;\n\t"
            "mul.wide.s32 w, %9, %11;\n\t"
            "mov.b64 {lo9, hi9}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.cc.u32 %6, lo6, hi5;\n\t"
            "addc.cc.u32 %7, lo7, hi6;\n\t"
            "addc.cc.u32 %8, lo8, hi7;\n\t"
            "addc.cc.u32 %9, lo9, hi8;\n\t"
            "addc.u32 %10, hi9, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "+r"(R[7]), "+r"(R[8]), "+r"(R[9]), "=r"(R[10])
            : "r"(y));
    }
};

template <>
struct MulWordS<11> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<11>, hi<11>;\n\t"
            "mul.wide.u32 w, %0, %12;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %12;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %12;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %12;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %12;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.u32 w, %5, %12;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mul.wide.u32 w, %6, %12;\n\t"
            "mov.b64 {lo6, hi6}, w;\n\t"
            "mul.wide.u32 w, %7, %12;\n\t"
            "mov.b64 {lo7, hi7}, w;\n\t"
            "mul.wide.u32 w, %8, %12;\n\t"
            "mov.b64 {lo8, hi8}, w;\n\t"
            "mul.wide.u32 w, %9, %12;\n\t"
            "mov.b64 {lo9, hi9}, w;\n\t"
            "mul.wide.s32 w, %10, %12;\n\t"
            "mov.b64 {lo10, hi10}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.cc.u32 %6, lo6, hi5;\n\t"
            "addc.cc.u32 %7, lo7, hi6;\n\t"
            "addc.cc.u32 %8, lo8, hi7;\n\t"
            "addc.cc.u32 %9, lo9, hi8;\n\t"
            "addc.cc.u32 %10, lo10, hi9;\n\t"
            "addc.u32 %11, hi10, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "+r"(R[7]), "+r"(R[8]), "+r"(R[9]), "+r"(R[10]), "=r"(R[11])
            : "r"(y));
    }
};

template <>
struct MulWordS<12> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<12>, hi<12>;\n\t"
            "mul.wide.u32 w, %0, %13;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %13;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %13;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %13;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %13;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.u32 w, %5, %13;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mul.wide.u32 w, %6, %13;\n\t"
            "mov.b64 {lo6, hi6}, w;\n\t"
            "mul.wide.u32 w, %7, %13;\n\t"
            "mov.b64 {lo7, hi7}, w;\n\t"
            "mul.wide.u32 w, %8, %13;\n\t"
            "mov.b64 {lo8, hi8}, w;\n\t"
            "mul.wide.u32 w, %9, %13;\n\t"
            "mov.b64 {lo9, hi9}, w;\n\t"
            "mul.wide.u32 w, %10, %13;\n\t"
            "mov.b64 {lo10, hi10}, w;\n\t"
            "mul.wide.s32 w, %11, %13;\n\t"
            "mov.b64 {lo11, hi11}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.cc.u32 %6, lo6, hi5;\n\t"
            "addc.cc.u32 %7, lo7, hi6;\n\t"
            "addc.cc.u32 %8, lo8, hi7;\n\t"
            "addc.cc.u32 %9, lo9, hi8;\n\t"
            "addc.cc.u32 %10, lo10, hi9;\n\t"
            "addc.cc.u32 %11, lo11, hi10;\n\t"
            "addc.u32 %12, hi11, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "+r"(R[7]), "+r"(R[8]), "+r"(R[9]), "+r"(R[10]), "+r"(R[11]), "=r"(R[12])
            : "r"(y));
    }
};

template <>
struct MulWordS<13> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<13>, hi<13>;\n\t"
            "mul.wide.u32 w, %0, %14;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %14;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %14;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %14;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %14;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.u32 w, %5, %14;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mul.wide.u32 w, %6, %14;\n\t"
            "mov.b64 {lo6, hi6}, w;\n\t"
            "mul.wide.u32 w, %7, %14;\n\t"
            "mov.b64 {lo7, hi7}, w;\n\t"
            "mul.wide.u32 w, %8, %14;\n\t"
            "mov.b64 {lo8, hi8}, w;\n\t"
            "mul.wide.u32 w, %9, %14;\n\t"
            "mov.b64 {lo9, hi9}, w;\n\t"
            "mul.wide.u32 w, %10, %14;\n\t"
            "mov.b64 {lo10, hi10}, w;\n\t"
            "mul.wide.u32 w, %11, %14;\n\t"
            "mov.b64 {lo11, hi11}, w;\n\t"
            "mul.wide.s32 w, %12, %14;\n\t"
            "mov.b64 {lo12, hi12}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.cc.u32 %6, lo6, hi5;\n\t"
            "addc.cc.u32 %7, lo7, hi6;\n\t"
            "addc.cc.u32 %8, lo8, hi7;\n\t"
            "addc.cc.u32 %9, lo9, hi8;\n\t"
            "addc.cc.u32 %10, lo10, hi9;\n\t"
            "addc.cc.u32 %11, lo11, hi10;\n\t"
            "addc.cc.u32 %12, lo12, hi11;\n\t"
            "addc.u32 %13, hi12, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "+r"(R[7]), "+r"(R[8]), "+r"(R[9]), "+r"(R[10]), "+r"(R[11]), "+r"(R[12]), "=r"(R[13])
            : "r"(y));
    }
};

template <>
struct MulWordS<14> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<14>, hi<14>;\n\t"
            "mul.wide.u32 w, %0, %15;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %15;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %15;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %15;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %15;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.u32 w, %5, %15;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mul.wide.u32 w, %6, %15;\n\t"
            "mov.b64 {lo6, hi6}, w;\n\t"
            "mul.wide.u32 w, %7, %15;\n\t"
            "mov.b64 {lo7, hi7}, w;\n\t"
            "mul.wide.u32 w, %8, %15;\n\t"
            "mov.b64 {lo8, hi8}, w;\n\t"
            "mul.wide.u32 w, %9, %15;\n\t"
            "mov.b64 {lo9, hi9}, w;\n\t"
            "mul.wide.u32 w, %10, %15;\n\t"
            "mov.b64 {lo10, hi10}, w;\n\t"
            "mul.wide.u32 w, %11, %15;\n\t"
            "mov.b64 {lo11, hi11}, w;\n\t"
            "mul.wide.u32 w, %12, %15;\n\t"
            "mov.b64 {lo12, hi12}, w;\n\t"
            "mul.wide.s32 w, %13, %15;\n\t"
            "mov.b64 {lo13, hi13}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.cc.u32 %6, lo6, hi5;\n\t"
            "addc.cc.u32 %7, lo7, hi6;\n\t"
            "addc.cc.u32 %8, lo8, hi7;\n\t"
            "addc.cc.u32 %9, lo9, hi8;\n\t"
            "addc.cc.u32 %10, lo10, hi9;\n\t"
            "addc.cc.u32 %11, lo11, hi10;\n\t"
            "addc.cc.u32 %12, lo12, hi11;\n\t"
            "addc.cc.u32 %13, lo13, hi12;\n\t"
            "addc.u32 %14, hi13, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "+r"(R[7]), "+r"(R[8]), "+r"(R[9]), "+r"(R[10]), "+r"(R[11]), "+r"(R[12]), "+r"(R[13]), "=r"(R[14])
            : "r"(y));
    }
};

template <>
struct MulWordS<15> {
    static __device__ __forceinline__ void apply(uint32_t *R, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<15>, hi<15>;\n\t"
            "mul.wide.u32 w, %0, %16;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %16;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %16;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %16;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mul.wide.u32 w, %4, %16;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mul.wide.u32 w, %5, %16;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mul.wide.u32 w, %6, %16;\n\t"
            "mov.b64 {lo6, hi6}, w;\n\t"
            "mul.wide.u32 w, %7, %16;\n\t"
            "mov.b64 {lo7, hi7}, w;\n\t"
            "mul.wide.u32 w, %8, %16;\n\t"
            "mov.b64 {lo8, hi8}, w;\n\t"
            "mul.wide.u32 w, %9, %16;\n\t"
            "mov.b64 {lo9, hi9}, w;\n\t"
            "mul.wide.u32 w, %10, %16;\n\t"
            "mov.b64 {lo10, hi10}, w;\n\t"
            "mul.wide.u32 w, %11, %16;\n\t"
            "mov.b64 {lo11, hi11}, w;\n\t"
            "mul.wide.u32 w, %12, %16;\n\t"
            "mov.b64 {lo12, hi12}, w;\n\t"
            "mul.wide.u32 w, %13, %16;\n\t"
            "mov.b64 {lo13, hi13}, w;\n\t"
            "mul.wide.s32 w, %14, %16;\n\t"
            "mov.b64 {lo14, hi14}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.cc.u32 %6, lo6, hi5;\n\t"
            "addc.cc.u32 %7, lo7, hi6;\n\t"
            "addc.cc.u32 %8, lo8, hi7;\n\t"
            "addc.cc.u32 %9, lo9, hi8;\n\t"
            "addc.cc.u32 %10, lo10, hi9;\n\t"
            "addc.cc.u32 %11, lo11, hi10;\n\t"
            "addc.cc.u32 %12, lo12, hi11;\n\t"
            "addc.cc.u32 %13, lo13, hi12;\n\t"
            "addc.cc.u32 %14, lo14, hi13;\n\t"
            "addc.u32 %15, hi14, 0;\n\t"
            "}"
            : "+r"(R[0]), "+r"(R[1]), "+r"(R[2]), "+r"(R[3]), "+r"(R[4]), "+r"(R[5]), "+r"(R[6]), "+r"(R[7]), "+r"(R[8]), "+r"(R[9]), "+r"(R[10]), "+r"(R[11]), "+r"(R[12]), "+r"(R[13]), "+r"(R[14]), "=r"(R[15])
            : "r"(y));
    }
};

// acc[0..NL-1] (two's complement) += sum_{l < NR-1} col[l] * 2^(32 l)
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

template <>
struct FoldCols<1, 2> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<1>, chi<1>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %2;\n\t"
            "shr.s32 ext, chi0, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.u32 %1, %1, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1])
            : "l"(colt));
    }
};

template <>
struct FoldCols<1, 3> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<1>, chi<1>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %3;\n\t"
            "shr.s32 ext, chi0, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, 0;\n\t"
            "addc.u32 %2, %2, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.u32 %2, %2, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2])
            : "l"(colt));
    }
};

template <>
struct FoldCols<1, 4> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<1>, chi<1>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %4;\n\t"
            "shr.s32 ext, chi0, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, 0;\n\t"
            "addc.cc.u32 %2, %2, 0;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, ext;\n\t"
            "addc.u32 %3, %3, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3])
            : "l"(colt));
    }
};

template <>
struct FoldCols<2, 3> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<2>, chi<2>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %3;\n\t"
            "mov.b64 {clo1, chi1}, %4;\n\t"
            "shr.s32 ext, chi1, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.u32 %2, %2, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.u32 %2, %2, chi1;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2])
            : "l"(col[0]), "l"(colt));
    }
};

template <>
struct FoldCols<2, 4> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<2>, chi<2>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %4;\n\t"
            "mov.b64 {clo1, chi1}, %5;\n\t"
            "shr.s32 ext, chi1, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, 0;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.u32 %3, %3, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3])
            : "l"(col[0]), "l"(colt));
    }
};

template <>
struct FoldCols<2, 5> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<2>, chi<2>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %5;\n\t"
            "mov.b64 {clo1, chi1}, %6;\n\t"
            "shr.s32 ext, chi1, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, 0;\n\t"
            "addc.cc.u32 %3, %3, 0;\n\t"
            "addc.u32 %4, %4, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, ext;\n\t"
            "addc.u32 %4, %4, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4])
            : "l"(col[0]), "l"(colt));
    }
};

template <>
struct FoldCols<3, 4> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<3>, chi<3>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %4;\n\t"
            "mov.b64 {clo1, chi1}, %5;\n\t"
            "mov.b64 {clo2, chi2}, %6;\n\t"
            "shr.s32 ext, chi2, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.u32 %3, %3, chi2;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3])
            : "l"(col[0]), "l"(col[1]), "l"(colt));
    }
};

template <>
struct FoldCols<3, 5> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<3>, chi<3>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %5;\n\t"
            "mov.b64 {clo1, chi1}, %6;\n\t"
            "mov.b64 {clo2, chi2}, %7;\n\t"
            "shr.s32 ext, chi2, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, 0;\n\t"
            "addc.u32 %4, %4, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.u32 %4, %4, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4])
            : "l"(col[0]), "l"(col[1]), "l"(colt));
    }
};

template <>
struct FoldCols<3, 6> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<3>, chi<3>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %6;\n\t"
            "mov.b64 {clo1, chi1}, %7;\n\t"
            "mov.b64 {clo2, chi2}, %8;\n\t"
            "shr.s32 ext, chi2, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, 0;\n\t"
            "addc.cc.u32 %4, %4, 0;\n\t"
            "addc.u32 %5, %5, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, ext;\n\t"
            "addc.u32 %5, %5, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5])
            : "l"(col[0]), "l"(col[1]), "l"(colt));
    }
};

template <>
struct FoldCols<4, 5> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<4>, chi<4>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %5;\n\t"
            "mov.b64 {clo1, chi1}, %6;\n\t"
            "mov.b64 {clo2, chi2}, %7;\n\t"
            "mov.b64 {clo3, chi3}, %8;\n\t"
            "shr.s32 ext, chi3, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.u32 %4, %4, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.u32 %4, %4, chi3;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(colt));
    }
};

template <>
struct FoldCols<4, 6> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<4>, chi<4>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %6;\n\t"
            "mov.b64 {clo1, chi1}, %7;\n\t"
            "mov.b64 {clo2, chi2}, %8;\n\t"
            "mov.b64 {clo3, chi3}, %9;\n\t"
            "shr.s32 ext, chi3, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, 0;\n\t"
            "addc.u32 %5, %5, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.u32 %5, %5, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(colt));
    }
};

template <>
struct FoldCols<4, 7> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<4>, chi<4>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %7;\n\t"
            "mov.b64 {clo1, chi1}, %8;\n\t"
            "mov.b64 {clo2, chi2}, %9;\n\t"
            "mov.b64 {clo3, chi3}, %10;\n\t"
            "shr.s32 ext, chi3, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, 0;\n\t"
            "addc.cc.u32 %5, %5, 0;\n\t"
            "addc.u32 %6, %6, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, ext;\n\t"
            "addc.u32 %6, %6, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(colt));
    }
};

template <>
struct FoldCols<5, 6> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<5>, chi<5>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %6;\n\t"
            "mov.b64 {clo1, chi1}, %7;\n\t"
            "mov.b64 {clo2, chi2}, %8;\n\t"
            "mov.b64 {clo3, chi3}, %9;\n\t"
            "mov.b64 {clo4, chi4}, %10;\n\t"
            "shr.s32 ext, chi4, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.u32 %5, %5, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.u32 %5, %5, chi4;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(colt));
    }
};

template <>
struct FoldCols<5, 7> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<5>, chi<5>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %7;\n\t"
            "mov.b64 {clo1, chi1}, %8;\n\t"
            "mov.b64 {clo2, chi2}, %9;\n\t"
            "mov.b64 {clo3, chi3}, %10;\n\t"
            "mov.b64 {clo4, chi4}, %11;\n\t"
            "shr.s32 ext, chi4, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, 0;\n\t"
            "addc.u32 %6, %6, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.u32 %6, %6, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(colt));
    }
};

template <>
struct FoldCols<5, 8> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<5>, chi<5>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %8;\n\t"
            "mov.b64 {clo1, chi1}, %9;\n\t"
            "mov.b64 {clo2, chi2}, %10;\n\t"
            "mov.b64 {clo3, chi3}, %11;\n\t"
            "mov.b64 {clo4, chi4}, %12;\n\t"
            "shr.s32 ext, chi4, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, 0;\n\t"
            "addc.cc.u32 %6, %6, 0;\n\t"
            "addc.u32 %7, %7, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, ext;\n\t"
            "addc.u32 %7, %7, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(colt));
    }
};

template <>
struct FoldCols<6, 7> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<6>, chi<6>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %7;\n\t"
            "mov.b64 {clo1, chi1}, %8;\n\t"
            "mov.b64 {clo2, chi2}, %9;\n\t"
            "mov.b64 {clo3, chi3}, %10;\n\t"
            "mov.b64 {clo4, chi4}, %11;\n\t"
            "mov.b64 {clo5, chi5}, %12;\n\t"
            "shr.s32 ext, chi5, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.u32 %6, %6, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.u32 %6, %6, chi5;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(colt));
    }
};

template <>
struct FoldCols<6, 8> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<6>, chi<6>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %8;\n\t"
            "mov.b64 {clo1, chi1}, %9;\n\t"
            "mov.b64 {clo2, chi2}, %10;\n\t"
            "mov.b64 {clo3, chi3}, %11;\n\t"
            "mov.b64 {clo4, chi4}, %12;\n\t"
            "mov.b64 {clo5, chi5}, %13;\n\t"
            "shr.s32 ext, chi5, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, 0;\n\t"
            "addc.u32 %7, %7, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.u32 %7, %7, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(colt));
    }
};

template <>
struct FoldCols<6, 9> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<6>, chi<6>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %9;\n\t"
            "mov.b64 {clo1, chi1}, %10;\n\t"
            "mov.b64 {clo2, chi2}, %11;\n\t"
            "mov.b64 {clo3, chi3}, %12;\n\t"
            "mov.b64 {clo4, chi4}, %13;\n\t"
            "mov.b64 {clo5, chi5}, %14;\n\t"
            "shr.s32 ext, chi5, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, 0;\n\t"
            "addc.cc.u32 %7, %7, 0;\n\t"
            "addc.u32 %8, %8, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, ext;\n\t"
            "addc.u32 %8, %8, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(colt));
    }
};

template <>
struct FoldCols<7, 8> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<7>, chi<7>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %8;\n\t"
            "mov.b64 {clo1, chi1}, %9;\n\t"
            "mov.b64 {clo2, chi2}, %10;\n\t"
            "mov.b64 {clo3, chi3}, %11;\n\t"
            "mov.b64 {clo4, chi4}, %12;\n\t"
            "mov.b64 {clo5, chi5}, %13;\n\t"
            "mov.b64 {clo6, chi6}, %14;\n\t"
            "shr.s32 ext, chi6, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.u32 %7, %7, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.u32 %7, %7, chi6;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(colt));
    }
};

template <>
struct FoldCols<7, 9> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<7>, chi<7>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %9;\n\t"
            "mov.b64 {clo1, chi1}, %10;\n\t"
            "mov.b64 {clo2, chi2}, %11;\n\t"
            "mov.b64 {clo3, chi3}, %12;\n\t"
            "mov.b64 {clo4, chi4}, %13;\n\t"
            "mov.b64 {clo5, chi5}, %14;\n\t"
            "mov.b64 {clo6, chi6}, %15;\n\t"
            "shr.s32 ext, chi6, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, 0;\n\t"
            "addc.u32 %8, %8, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.u32 %8, %8, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(colt));
    }
};

template <>
struct FoldCols<7, 10> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<7>, chi<7>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %10;\n\t"
            "mov.b64 {clo1, chi1}, %11;\n\t"
            "mov.b64 {clo2, chi2}, %12;\n\t"
            "mov.b64 {clo3, chi3}, %13;\n\t"
            "mov.b64 {clo4, chi4}, %14;\n\t"
            "mov.b64 {clo5, chi5}, %15;\n\t"
            "mov.b64 {clo6, chi6}, %16;\n\t"
            "shr.s32 ext, chi6, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, 0;\n\t"
            "addc.cc.u32 %8, %8, 0;\n\t"
            "addc.u32 %9, %9, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, ext;\n\t"
            "addc.u32 %9, %9, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(colt));
    }
};

template <>
struct FoldCols<8, 9> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<8>, chi<8>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %9;\n\t"
            "mov.b64 {clo1, chi1}, %10;\n\t"
            "mov.b64 {clo2, chi2}, %11;\n\t"
            "mov.b64 {clo3, chi3}, %12;\n\t"
            "mov.b64 {clo4, chi4}, %13;\n\t"
            "mov.b64 {clo5, chi5}, %14;\n\t"
            "mov.b64 {clo6, chi6}, %15;\n\t"
            "mov.b64 {clo7, chi7}, %16;\n\t"
            "shr.s32 ext, chi7, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.u32 %8, %8, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.u32 %8, %8, chi7;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(colt));
    }
};

template <>
struct FoldCols<8, 10> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<8>, chi<8>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %10;\n\t"
            "mov.b64 {clo1, chi1}, %11;\n\t"
            "mov.b64 {clo2, chi2}, %12;\n\t"
            "mov.b64 {clo3, chi3}, %13;\n\t"
            "mov.b64 {clo4, chi4}, %14;\n\t"
            "mov.b64 {clo5, chi5}, %15;\n\t"
            "mov.b64 {clo6, chi6}, %16;\n\t"
            "mov.b64 {clo7, chi7}, %17;\n\t"
            "shr.s32 ext, chi7, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, 0;\n\t"
            "addc.u32 %9, %9, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.u32 %9, %9, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(colt));
    }
};

template <>
struct FoldCols<8, 11> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<8>, chi<8>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %11;\n\t"
            "mov.b64 {clo1, chi1}, %12;\n\t"
            "mov.b64 {clo2, chi2}, %13;\n\t"
            "mov.b64 {clo3, chi3}, %14;\n\t"
            "mov.b64 {clo4, chi4}, %15;\n\t"
            "mov.b64 {clo5, chi5}, %16;\n\t"
            "mov.b64 {clo6, chi6}, %17;\n\t"
            "mov.b64 {clo7, chi7}, %18;\n\t"
            "shr.s32 ext, chi7, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, 0;\n\t"
            "addc.cc.u32 %9, %9, 0;\n\t"
            "addc.u32 %10, %10, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, ext;\n\t"
            "addc.u32 %10, %10, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(colt));
    }
};

template <>
struct FoldCols<9, 10> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<9>, chi<9>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %10;\n\t"
            "mov.b64 {clo1, chi1}, %11;\n\t"
            "mov.b64 {clo2, chi2}, %12;\n\t"
            "mov.b64 {clo3, chi3}, %13;\n\t"
            "mov.b64 {clo4, chi4}, %14;\n\t"
            "mov.b64 {clo5, chi5}, %15;\n\t"
            "mov.b64 {clo6, chi6}, %16;\n\t"
            "mov.b64 {clo7, chi7}, %17;\n\t"
            "mov.b64 {clo8, chi8}, %18;\n\t"
            "shr.s32 ext, chi8, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.u32 %9, %9, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.u32 %9, %9, chi8;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(colt));
    }
};

template <>
struct FoldCols<9, 11> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<9>, chi<9>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %11;\n\t"
            "mov.b64 {clo1, chi1}, %12;\n\t"
            "mov.b64 {clo2, chi2}, %13;\n\t"
            "mov.b64 {clo3, chi3}, %14;\n\t"
            "mov.b64 {clo4, chi4}, %15;\n\t"
            "mov.b64 {clo5, chi5}, %16;\n\t"
            "mov.b64 {clo6, chi6}, %17;\n\t"
            "mov.b64 {clo7, chi7}, %18;\n\t"
            "mov.b64 {clo8, chi8}, %19;\n\t"
            "shr.s32 ext, chi8, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, 0;\n\t"
            "addc.u32 %10, %10, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.u32 %10, %10, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(colt));
    }
};

template <>
struct FoldCols<9, 12> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<9>, chi<9>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %12;\n\t"
            "mov.b64 {clo1, chi1}, %13;\n\t"
            "mov.b64 {clo2, chi2}, %14;\n\t"
            "mov.b64 {clo3, chi3}, %15;\n\t"
            "mov.b64 {clo4, chi4}, %16;\n\t"
            "mov.b64 {clo5, chi5}, %17;\n\t"
            "mov.b64 {clo6, chi6}, %18;\n\t"
            "mov.b64 {clo7, chi7}, %19;\n\t"
            "mov.b64 {clo8, chi8}, %20;\n\t"
            "shr.s32 ext, chi8, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, 0;\n\t"
            "addc.cc.u32 %10, %10, 0;\n\t"
            "addc.u32 %11, %11, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, ext;\n\t"
            "addc.u32 %11, %11, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(colt));
    }
};

template <>
struct FoldCols<10, 11> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<10>, chi<10>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %11;\n\t"
            "mov.b64 {clo1, chi1}, %12;\n\t"
            "mov.b64 {clo2, chi2}, %13;\n\t"
            "mov.b64 {clo3, chi3}, %14;\n\t"
            "mov.b64 {clo4, chi4}, %15;\n\t"
            "mov.b64 {clo5, chi5}, %16;\n\t"
            "mov.b64 {clo6, chi6}, %17;\n\t"
            "mov.b64 {clo7, chi7}, %18;\n\t"
            "mov.b64 {clo8, chi8}, %19;\n\t"
            "mov.b64 {clo9, chi9}, %20;\n\t"
            "shr.s32 ext, chi9, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.u32 %10, %10, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.u32 %10, %10, chi9;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(colt));
    }
};

template <>
struct FoldCols<10, 12> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<10>, chi<10>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %12;\n\t"
            "mov.b64 {clo1, chi1}, %13;\n\t"
            "mov.b64 {clo2, chi2}, %14;\n\t"
            "mov.b64 {clo3, chi3}, %15;\n\t"
            "mov.b64 {clo4, chi4}, %16;\n\t"
            "mov.b64 {clo5, chi5}, %17;\n\t"
            "mov.b64 {clo6, chi6}, %18;\n\t"
            "mov.b64 {clo7, chi7}, %19;\n\t"
            "mov.b64 {clo8, chi8}, %20;\n\t"
            "mov.b64 {clo9, chi9}, %21;\n\t"
            "shr.s32 ext, chi9, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, 0;\n\t"
            "addc.u32 %11, %11, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.u32 %11, %11, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(colt));
    }
};

template <>
struct FoldCols<10, 13> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<10>, chi<10>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %13;\n\t"
            "mov.b64 {clo1, chi1}, %14;\n\t"
            "mov.b64 {clo2, chi2}, %15;\n\t"
            "mov.b64 {clo3, chi3}, %16;\n\t"
            "mov.b64 {clo4, chi4}, %17;\n\t"
            "mov.b64 {clo5, chi5}, %18;\n\t"
            "mov.b64 {clo6, chi6}, %19;\n\t"
            "mov.b64 {clo7, chi7}, %20;\n\t"
            "mov.b64 {clo8, chi8}, %21;\n\t"
            "mov.b64 {clo9, chi9}, %22;\n\t"
            "shr.s32 ext, chi9, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, 0;\n\t"
            "addc.cc.u32 %11, %11, 0;\n\t"
            "addc.u32 %12, %12, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, ext;\n\t"
            "addc.u32 %12, %12, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(colt));
    }
};

template <>
struct FoldCols<11, 12> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<11>, chi<11>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %12;\n\t"
            "mov.b64 {clo1, chi1}, %13;\n\t"
            "mov.b64 {clo2, chi2}, %14;\n\t"
            "mov.b64 {clo3, chi3}, %15;\n\t"
            "mov.b64 {clo4, chi4}, %16;\n\t"
            "mov.b64 {clo5, chi5}, %17;\n\t"
            "mov.b64 {clo6, chi6}, %18;\n\t"
            "mov.b64 {clo7, chi7}, %19;\n\t"
            "mov.b64 {clo8, chi8}, %20;\n\t"
            "mov.b64 {clo9, chi9}, %21;\n\t"
            "mov.b64 {clo10, chi10}, %22;\n\t"
            "shr.s32 ext, chi10, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.u32 %11, %11, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.u32 %11, %11, chi10;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(colt));
    }
};

template <>
struct FoldCols<11, 13> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<11>, chi<11>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %13;\n\t"
            "mov.b64 {clo1, chi1}, %14;\n\t"
            "mov.b64 {clo2, chi2}, %15;\n\t"
            "mov.b64 {clo3, chi3}, %16;\n\t"
            "mov.b64 {clo4, chi4}, %17;\n\t"
            "mov.b64 {clo5, chi5}, %18;\n\t"
            "mov.b64 {clo6, chi6}, %19;\n\t"
            "mov.b64 {clo7, chi7}, %20;\n\t"
            "mov.b64 {clo8, chi8}, %21;\n\t"
            "mov.b64 {clo9, chi9}, %22;\n\t"
            "mov.b64 {clo10, chi10}, %23;\n\t"
            "shr.s32 ext, chi10, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, 0;\n\t"
            "addc.u32 %12, %12, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.u32 %12, %12, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(colt));
    }
};

template <>
struct FoldCols<11, 14> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<11>, chi<11>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %14;\n\t"
            "mov.b64 {clo1, chi1}, %15;\n\t"
            "mov.b64 {clo2, chi2}, %16;\n\t"
            "mov.b64 {clo3, chi3}, %17;\n\t"
            "mov.b64 {clo4, chi4}, %18;\n\t"
            "mov.b64 {clo5, chi5}, %19;\n\t"
            "mov.b64 {clo6, chi6}, %20;\n\t"
            "mov.b64 {clo7, chi7}, %21;\n\t"
            "mov.b64 {clo8, chi8}, %22;\n\t"
            "mov.b64 {clo9, chi9}, %23;\n\t"
            "mov.b64 {clo10, chi10}, %24;\n\t"
            "shr.s32 ext, chi10, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, 0;\n\t"
            "addc.cc.u32 %12, %12, 0;\n\t"
            "addc.u32 %13, %13, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.cc.u32 %12, %12, ext;\n\t"
            "addc.u32 %13, %13, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12]), "+r"(acc[13])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(colt));
    }
};

template <>
struct FoldCols<12, 13> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<12>, chi<12>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %13;\n\t"
            "mov.b64 {clo1, chi1}, %14;\n\t"
            "mov.b64 {clo2, chi2}, %15;\n\t"
            "mov.b64 {clo3, chi3}, %16;\n\t"
            "mov.b64 {clo4, chi4}, %17;\n\t"
            "mov.b64 {clo5, chi5}, %18;\n\t"
            "mov.b64 {clo6, chi6}, %19;\n\t"
            "mov.b64 {clo7, chi7}, %20;\n\t"
            "mov.b64 {clo8, chi8}, %21;\n\t"
            "mov.b64 {clo9, chi9}, %22;\n\t"
            "mov.b64 {clo10, chi10}, %23;\n\t"
            "mov.b64 {clo11, chi11}, %24;\n\t"
            "shr.s32 ext, chi11, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, clo11;\n\t"
            "addc.u32 %12, %12, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.u32 %12, %12, chi11;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(col[10]), "l"(colt));
    }
};

template <>
struct FoldCols<12, 14> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<12>, chi<12>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %14;\n\t"
            "mov.b64 {clo1, chi1}, %15;\n\t"
            "mov.b64 {clo2, chi2}, %16;\n\t"
            "mov.b64 {clo3, chi3}, %17;\n\t"
            "mov.b64 {clo4, chi4}, %18;\n\t"
            "mov.b64 {clo5, chi5}, %19;\n\t"
            "mov.b64 {clo6, chi6}, %20;\n\t"
            "mov.b64 {clo7, chi7}, %21;\n\t"
            "mov.b64 {clo8, chi8}, %22;\n\t"
            "mov.b64 {clo9, chi9}, %23;\n\t"
            "mov.b64 {clo10, chi10}, %24;\n\t"
            "mov.b64 {clo11, chi11}, %25;\n\t"
            "shr.s32 ext, chi11, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, clo11;\n\t"
            "addc.cc.u32 %12, %12, 0;\n\t"
            "addc.u32 %13, %13, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.cc.u32 %12, %12, chi11;\n\t"
            "addc.u32 %13, %13, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12]), "+r"(acc[13])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(col[10]), "l"(colt));
    }
};

template <>
struct FoldCols<12, 15> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<12>, chi<12>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %15;\n\t"
            "mov.b64 {clo1, chi1}, %16;\n\t"
            "mov.b64 {clo2, chi2}, %17;\n\t"
            "mov.b64 {clo3, chi3}, %18;\n\t"
            "mov.b64 {clo4, chi4}, %19;\n\t"
            "mov.b64 {clo5, chi5}, %20;\n\t"
            "mov.b64 {clo6, chi6}, %21;\n\t"
            "mov.b64 {clo7, chi7}, %22;\n\t"
            "mov.b64 {clo8, chi8}, %23;\n\t"
            "mov.b64 {clo9, chi9}, %24;\n\t"
            "mov.b64 {clo10, chi10}, %25;\n\t"
            "mov.b64 {clo11, chi11}, %26;\n\t"
            "shr.s32 ext, chi11, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, clo11;\n\t"
            "addc.cc.u32 %12, %12, 0;\n\t"
            "addc.cc.u32 %13, %13, 0;\n\t"
            "addc.u32 %14, %14, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.cc.u32 %12, %12, chi11;\n\t"
            "addc.cc.u32 %13, %13, ext;\n\t"
            "addc.u32 %14, %14, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12]), "+r"(acc[13]), "+r"(acc[14])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(col[10]), "l"(colt));
    }
};

template <>
struct FoldCols<13, 14> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<13>, chi<13>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %14;\n\t"
            "mov.b64 {clo1, chi1}, %15;\n\t"
            "mov.b64 {clo2, chi2}, %16;\n\t"
            "mov.b64 {clo3, chi3}, %17;\n\t"
            "mov.b64 {clo4, chi4}, %18;\n\t"
            "mov.b64 {clo5, chi5}, %19;\n\t"
            "mov.b64 {clo6, chi6}, %20;\n\t"
            "mov.b64 {clo7, chi7}, %21;\n\t"
            "mov.b64 {clo8, chi8}, %22;\n\t"
            "mov.b64 {clo9, chi9}, %23;\n\t"
            "mov.b64 {clo10, chi10}, %24;\n\t"
            "mov.b64 {clo11, chi11}, %25;\n\t"
            "mov.b64 {clo12, chi12}, %26;\n\t"
            "shr.s32 ext, chi12, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, clo11;\n\t"
            "addc.cc.u32 %12, %12, clo12;\n\t"
            "addc.u32 %13, %13, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.cc.u32 %12, %12, chi11;\n\t"
            "addc.u32 %13, %13, chi12;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12]), "+r"(acc[13])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(col[10]), "l"(col[11]), "l"(colt));
    }
};

template <>
struct FoldCols<13, 15> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<13>, chi<13>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %15;\n\t"
            "mov.b64 {clo1, chi1}, %16;\n\t"
            "mov.b64 {clo2, chi2}, %17;\n\t"
            "mov.b64 {clo3, chi3}, %18;\n\t"
            "mov.b64 {clo4, chi4}, %19;\n\t"
            "mov.b64 {clo5, chi5}, %20;\n\t"
            "mov.b64 {clo6, chi6}, %21;\n\t"
            "mov.b64 {clo7, chi7}, %22;\n\t"
            "mov.b64 {clo8, chi8}, %23;\n\t"
            "mov.b64 {clo9, chi9}, %24;\n\t"
            "mov.b64 {clo10, chi10}, %25;\n\t"
            "mov.b64 {clo11, chi11}, %26;\n\t"
            "mov.b64 {clo12, chi12}, %27;\n\t"
            "shr.s32 ext, chi12, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, clo11;\n\t"
            "addc.cc.u32 %12, %12, clo12;\n\t"
            "addc.cc.u32 %13, %13, 0;\n\t"
            "addc.u32 %14, %14, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.cc.u32 %12, %12, chi11;\n\t"
            "addc.cc.u32 %13, %13, chi12;\n\t"
            "addc.u32 %14, %14, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12]), "+r"(acc[13]), "+r"(acc[14])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(col[10]), "l"(col[11]), "l"(colt));
    }
};

template <>
struct FoldCols<13, 16> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<13>, chi<13>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %16;\n\t"
            "mov.b64 {clo1, chi1}, %17;\n\t"
            "mov.b64 {clo2, chi2}, %18;\n\t"
            "mov.b64 {clo3, chi3}, %19;\n\t"
            "mov.b64 {clo4, chi4}, %20;\n\t"
            "mov.b64 {clo5, chi5}, %21;\n\t"
            "mov.b64 {clo6, chi6}, %22;\n\t"
            "mov.b64 {clo7, chi7}, %23;\n\t"
            "mov.b64 {clo8, chi8}, %24;\n\t"
            "mov.b64 {clo9, chi9}, %25;\n\t"
            "mov.b64 {clo10, chi10}, %26;\n\t"
            "mov.b64 {clo11, chi11}, %27;\n\t"
            "mov.b64 {clo12, chi12}, %28;\n\t"
            "shr.s32 ext, chi12, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, clo11;\n\t"
            "addc.cc.u32 %12, %12, clo12;\n\t"
            "addc.cc.u32 %13, %13, 0;\n\t"
            "addc.cc.u32 %14, %14, 0;\n\t"
            "addc.u32 %15, %15, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.cc.u32 %12, %12, chi11;\n\t"
            "addc.cc.u32 %13, %13, chi12;\n\t"
            "addc.cc.u32 %14, %14, ext;\n\t"
            "addc.u32 %15, %15, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12]), "+r"(acc[13]), "+r"(acc[14]), "+r"(acc[15])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(col[10]), "l"(col[11]), "l"(colt));
    }
};

template <>
struct FoldCols<14, 15> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<14>, chi<14>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %15;\n\t"
            "mov.b64 {clo1, chi1}, %16;\n\t"
            "mov.b64 {clo2, chi2}, %17;\n\t"
            "mov.b64 {clo3, chi3}, %18;\n\t"
            "mov.b64 {clo4, chi4}, %19;\n\t"
            "mov.b64 {clo5, chi5}, %20;\n\t"
            "mov.b64 {clo6, chi6}, %21;\n\t"
            "mov.b64 {clo7, chi7}, %22;\n\t"
            "mov.b64 {clo8, chi8}, %23;\n\t"
            "mov.b64 {clo9, chi9}, %24;\n\t"
            "mov.b64 {clo10, chi10}, %25;\n\t"
            "mov.b64 {clo11, chi11}, %26;\n\t"
            "mov.b64 {clo12, chi12}, %27;\n\t"
            "mov.b64 {clo13, chi13}, %28;\n\t"
            "shr.s32 ext, chi13, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, clo11;\n\t"
            "addc.cc.u32 %12, %12, clo12;\n\t"
            "addc.cc.u32 %13, %13, clo13;\n\t"
            "addc.u32 %14, %14, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.cc.u32 %12, %12, chi11;\n\t"
            "addc.cc.u32 %13, %13, chi12;\n\t"
            "addc.u32 %14, %14, chi13;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12]), "+r"(acc[13]), "+r"(acc[14])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(col[10]), "l"(col[11]), "l"(col[12]), "l"(colt));
    }
};

template <>
struct FoldCols<14, 16> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<14>, chi<14>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %16;\n\t"
            "mov.b64 {clo1, chi1}, %17;\n\t"
            "mov.b64 {clo2, chi2}, %18;\n\t"
            "mov.b64 {clo3, chi3}, %19;\n\t"
            "mov.b64 {clo4, chi4}, %20;\n\t"
            "mov.b64 {clo5, chi5}, %21;\n\t"
            "mov.b64 {clo6, chi6}, %22;\n\t"
            "mov.b64 {clo7, chi7}, %23;\n\t"
            "mov.b64 {clo8, chi8}, %24;\n\t"
            "mov.b64 {clo9, chi9}, %25;\n\t"
            "mov.b64 {clo10, chi10}, %26;\n\t"
            "mov.b64 {clo11, chi11}, %27;\n\t"
            "mov.b64 {clo12, chi12}, %28;\n\t"
            "mov.b64 {clo13, chi13}, %29;\n\t"
            "shr.s32 ext, chi13, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, clo11;\n\t"
            "addc.cc.u32 %12, %12, clo12;\n\t"
            "addc.cc.u32 %13, %13, clo13;\n\t"
            "addc.cc.u32 %14, %14, 0;\n\t"
            "addc.u32 %15, %15, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.cc.u32 %12, %12, chi11;\n\t"
            "addc.cc.u32 %13, %13, chi12;\n\t"
            "addc.cc.u32 %14, %14, chi13;\n\t"
            "addc.u32 %15, %15, ext;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12]), "+r"(acc[13]), "+r"(acc[14]), "+r"(acc[15])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(col[10]), "l"(col[11]), "l"(col[12]), "l"(colt));
    }
};

template <>
struct FoldCols<15, 16> {
    static __device__ __forceinline__ void apply(uint32_t *acc, const uint64_t *col, int64_t colt) {
        asm("{\n\t"
            ".reg .u32 clo<15>, chi<15>, ext;\n\t"
            "mov.b64 {clo0, chi0}, %16;\n\t"
            "mov.b64 {clo1, chi1}, %17;\n\t"
            "mov.b64 {clo2, chi2}, %18;\n\t"
            "mov.b64 {clo3, chi3}, %19;\n\t"
            "mov.b64 {clo4, chi4}, %20;\n\t"
            "mov.b64 {clo5, chi5}, %21;\n\t"
            "mov.b64 {clo6, chi6}, %22;\n\t"
            "mov.b64 {clo7, chi7}, %23;\n\t"
            "mov.b64 {clo8, chi8}, %24;\n\t"
            "mov.b64 {clo9, chi9}, %25;\n\t"
            "mov.b64 {clo10, chi10}, %26;\n\t"
            "mov.b64 {clo11, chi11}, %27;\n\t"
            "mov.b64 {clo12, chi12}, %28;\n\t"
            "mov.b64 {clo13, chi13}, %29;\n\t"
            "mov.b64 {clo14, chi14}, %30;\n\t"
            "shr.s32 ext, chi14, 31;\n\t"
            "add.cc.u32 %0, %0, clo0;\n\t"
            "addc.cc.u32 %1, %1, clo1;\n\t"
            "addc.cc.u32 %2, %2, clo2;\n\t"
            "addc.cc.u32 %3, %3, clo3;\n\t"
            "addc.cc.u32 %4, %4, clo4;\n\t"
            "addc.cc.u32 %5, %5, clo5;\n\t"
            "addc.cc.u32 %6, %6, clo6;\n\t"
            "addc.cc.u32 %7, %7, clo7;\n\t"
            "addc.cc.u32 %8, %8, clo8;\n\t"
            "addc.cc.u32 %9, %9, clo9;\n\t"
            "addc.cc.u32 %10, %10, clo10;\n\t"
            "addc.cc.u32 %11, %11, clo11;\n\t"
            "addc.cc.u32 %12, %12, clo12;\n\t"
            "addc.cc.u32 %13, %13, clo13;\n\t"
            "addc.cc.u32 %14, %14, clo14;\n\t"
            "addc.u32 %15, %15, 0;\n\t"
            "add.cc.u32 %1, %1, chi0;\n\t"
            "addc.cc.u32 %2, %2, chi1;\n\t"
            "addc.cc.u32 %3, %3, chi2;\n\t"
            "addc.cc.u32 %4, %4, chi3;\n\t"
            "addc.cc.u32 %5, %5, chi4;\n\t"
            "addc.cc.u32 %6, %6, chi5;\n\t"
            "addc.cc.u32 %7, %7, chi6;\n\t"
            "addc.cc.u32 %8, %8, chi7;\n\t"
            "addc.cc.u32 %9, %9, chi8;\n\t"
            "addc.cc.u32 %10, %10, chi9;\n\t"
            "addc.cc.u32 %11, %11, chi10;\n\t"
            "addc.cc.u32 %12, %12, chi11;\n\t"
            "addc.cc.u32 %13, %13, chi12;\n\t"
            "addc.cc.u32 %14, %14, chi13;\n\t"
            "addc.u32 %15, %15, chi14;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12]), "+r"(acc[13]), "+r"(acc[14]), "+r"(acc[15])
            : "l"(col[0]), "l"(col[1]), "l"(col[2]), "l"(col[3]), "l"(col[4]), "l"(col[5]), "l"(col[6]), "l"(col[7]), "l"(col[8]), "l"(col[9]), "l"(col[10]), "l"(col[11]), "l"(col[12]), "l"(col[13]), "l"(colt));
    }
};

}  // namespace pg
