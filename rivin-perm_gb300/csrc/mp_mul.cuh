// Multi-word by one-word multiplication for the exact Glynn product:
//   P[0..L] = P[0..L-1] * y   (unsigned, little-endian 32-bit words)
// as L independent mul.wide.u32 products (IMAD pipe) followed by one
// add.cc/addc carry chain over their halves (ALU pipe), so no 64-bit
// addend has to be assembled in a register pair.  Generated for L <= 15.
#pragma once
#include <stdint.h>

namespace pg {

template <int L>
struct MulWord {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
        uint32_t carry = 0;
#pragma unroll
        for (int l = 0; l < L; l++) {
            const uint64_t t = (uint64_t)P[l] * y + carry;
            P[l] = (uint32_t)t;
            carry = (uint32_t)(t >> 32);
        }
        P[L] = carry;
    }
};

template <>
struct MulWord<1> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<1>, hi<1>;\n\t"
            "mul.wide.u32 w, %0, %2;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "mov.b32 %1, hi0;\n\t"
            "}"
            : "+r"(P[0]), "=r"(P[1])
            : "r"(y));
    }
};

template <>
struct MulWord<2> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<2>, hi<2>;\n\t"
            "mul.wide.u32 w, %0, %3;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %3;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.u32 %2, hi1, 0;\n\t"
            "}"
            : "+r"(P[0]), "+r"(P[1]), "=r"(P[2])
            : "r"(y));
    }
};

template <>
struct MulWord<3> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<3>, hi<3>;\n\t"
            "mul.wide.u32 w, %0, %4;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %4;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %4;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.u32 %3, hi2, 0;\n\t"
            "}"
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "=r"(P[3])
            : "r"(y));
    }
};

template <>
struct MulWord<4> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 lo<4>, hi<4>;\n\t"
            "mul.wide.u32 w, %0, %5;\n\t"
            "mov.b64 {lo0, hi0}, w;\n\t"
            "mul.wide.u32 w, %1, %5;\n\t"
            "mov.b64 {lo1, hi1}, w;\n\t"
            "mul.wide.u32 w, %2, %5;\n\t"
            "mov.b64 {lo2, hi2}, w;\n\t"
            "mul.wide.u32 w, %3, %5;\n\t"
            "mov.b64 {lo3, hi3}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.u32 %4, hi3, 0;\n\t"
            "}"
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "=r"(P[4])
            : "r"(y));
    }
};

template <>
struct MulWord<5> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %4, %6;\n\t"
            "mov.b64 {lo4, hi4}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.u32 %5, hi4, 0;\n\t"
            "}"
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "=r"(P[5])
            : "r"(y));
    }
};

template <>
struct MulWord<6> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %5, %7;\n\t"
            "mov.b64 {lo5, hi5}, w;\n\t"
            "mov.b32 %0, lo0;\n\t"
            "add.cc.u32 %1, lo1, hi0;\n\t"
            "addc.cc.u32 %2, lo2, hi1;\n\t"
            "addc.cc.u32 %3, lo3, hi2;\n\t"
            "addc.cc.u32 %4, lo4, hi3;\n\t"
            "addc.cc.u32 %5, lo5, hi4;\n\t"
            "addc.u32 %6, hi5, 0;\n\t"
            "}"
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "=r"(P[6])
            : "r"(y));
    }
};

template <>
struct MulWord<7> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %6, %8;\n\t"
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
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "+r"(P[6]), "=r"(P[7])
            : "r"(y));
    }
};

template <>
struct MulWord<8> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %7, %9;\n\t"
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
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "+r"(P[6]), "+r"(P[7]), "=r"(P[8])
            : "r"(y));
    }
};

template <>
struct MulWord<9> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %8, %10;\n\t"
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
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "+r"(P[6]), "+r"(P[7]), "+r"(P[8]), "=r"(P[9])
            : "r"(y));
    }
};

template <>
struct MulWord<10> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %9, %11;\n\t"
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
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "+r"(P[6]), "+r"(P[7]), "+r"(P[8]), "+r"(P[9]), "=r"(P[10])
            : "r"(y));
    }
};

template <>
struct MulWord<11> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %10, %12;\n\t"
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
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "+r"(P[6]), "+r"(P[7]), "+r"(P[8]), "+r"(P[9]), "+r"(P[10]), "=r"(P[11])
            : "r"(y));
    }
};

template <>
struct MulWord<12> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %11, %13;\n\t"
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
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "+r"(P[6]), "+r"(P[7]), "+r"(P[8]), "+r"(P[9]), "+r"(P[10]), "+r"(P[11]), "=r"(P[12])
            : "r"(y));
    }
};

template <>
struct MulWord<13> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %12, %14;\n\t"
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
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "+r"(P[6]), "+r"(P[7]), "+r"(P[8]), "+r"(P[9]), "+r"(P[10]), "+r"(P[11]), "+r"(P[12]), "=r"(P[13])
            : "r"(y));
    }
};

template <>
struct MulWord<14> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %13, %15;\n\t"
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
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "+r"(P[6]), "+r"(P[7]), "+r"(P[8]), "+r"(P[9]), "+r"(P[10]), "+r"(P[11]), "+r"(P[12]), "+r"(P[13]), "=r"(P[14])
            : "r"(y));
    }
};

template <>
struct MulWord<15> {
    static __device__ __forceinline__ void apply(uint32_t *P, uint32_t y) {
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
            "mul.wide.u32 w, %14, %16;\n\t"
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
            : "+r"(P[0]), "+r"(P[1]), "+r"(P[2]), "+r"(P[3]), "+r"(P[4]), "+r"(P[5]), "+r"(P[6]), "+r"(P[7]), "+r"(P[8]), "+r"(P[9]), "+r"(P[10]), "+r"(P[11]), "+r"(P[12]), "+r"(P[13]), "+r"(P[14]), "=r"(P[15])
            : "r"(y));
    }
};

}  // namespace pg
