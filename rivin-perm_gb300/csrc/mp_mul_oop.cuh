// Out-of-place variant of MulWord: Q[0..L] = P[0..L-1] * y with fresh
// output registers (lets the register allocator place each product half
// directly, without moving it into the input's register).
#pragma once
#include <stdint.h>

namespace pg {

template <int L>
struct MulWordOop {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        uint32_t carry = 0;
#pragma unroll
        for (int l = 0; l < L; l++) {
            const uint64_t t = (uint64_t)P[l] * y + carry;
            Q[l] = (uint32_t)t;
            carry = (uint32_t)(t >> 32);
        }
        Q[L] = carry;
    }
};

template <>
struct MulWordOop<1> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<1>;\n\t"
            "mul.wide.u32 w, %2, %3;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mov.b32 %1, hi0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1])
            : "r"(P[0]), "r"(y));
    }
};

template <>
struct MulWordOop<2> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<2>;\n\t"
            "mul.wide.u32 w, %3, %5;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %4, %5;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.u32 %2, hi1, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2])
            : "r"(P[0]), "r"(P[1]), "r"(y));
    }
};

template <>
struct MulWordOop<3> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<3>;\n\t"
            "mul.wide.u32 w, %4, %7;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %5, %7;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %6, %7;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.u32 %3, hi2, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(y));
    }
};

template <>
struct MulWordOop<4> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<4>;\n\t"
            "mul.wide.u32 w, %5, %9;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %6, %9;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %7, %9;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %8, %9;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.u32 %4, hi3, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(y));
    }
};

template <>
struct MulWordOop<5> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<5>;\n\t"
            "mul.wide.u32 w, %6, %11;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %7, %11;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %8, %11;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %9, %11;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %10, %11;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.u32 %5, hi4, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(y));
    }
};

template <>
struct MulWordOop<6> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<6>;\n\t"
            "mul.wide.u32 w, %7, %13;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %8, %13;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %9, %13;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %10, %13;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %11, %13;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %12, %13;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.u32 %6, hi5, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(y));
    }
};

template <>
struct MulWordOop<7> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<7>;\n\t"
            "mul.wide.u32 w, %8, %15;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %9, %15;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %10, %15;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %11, %15;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %12, %15;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %13, %15;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "mul.wide.u32 w, %14, %15;\n\t"
            "mov.b64 {%6, hi6}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.cc.u32 %6, %6, hi5;\n\t"
            "addc.u32 %7, hi6, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6]), "=&r"(Q[7])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(y));
    }
};

template <>
struct MulWordOop<8> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<8>;\n\t"
            "mul.wide.u32 w, %9, %17;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %10, %17;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %11, %17;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %12, %17;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %13, %17;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %14, %17;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "mul.wide.u32 w, %15, %17;\n\t"
            "mov.b64 {%6, hi6}, w;\n\t"
            "mul.wide.u32 w, %16, %17;\n\t"
            "mov.b64 {%7, hi7}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.cc.u32 %6, %6, hi5;\n\t"
            "addc.cc.u32 %7, %7, hi6;\n\t"
            "addc.u32 %8, hi7, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6]), "=&r"(Q[7]), "=&r"(Q[8])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(y));
    }
};

template <>
struct MulWordOop<9> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<9>;\n\t"
            "mul.wide.u32 w, %10, %19;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %11, %19;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %12, %19;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %13, %19;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %14, %19;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %15, %19;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "mul.wide.u32 w, %16, %19;\n\t"
            "mov.b64 {%6, hi6}, w;\n\t"
            "mul.wide.u32 w, %17, %19;\n\t"
            "mov.b64 {%7, hi7}, w;\n\t"
            "mul.wide.u32 w, %18, %19;\n\t"
            "mov.b64 {%8, hi8}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.cc.u32 %6, %6, hi5;\n\t"
            "addc.cc.u32 %7, %7, hi6;\n\t"
            "addc.cc.u32 %8, %8, hi7;\n\t"
            "addc.u32 %9, hi8, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6]), "=&r"(Q[7]), "=&r"(Q[8]), "=&r"(Q[9])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(y));
    }
};

template <>
struct MulWordOop<10> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<10>;\n\t"
            "mul.wide.u32 w, %11, %21;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %12, %21;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %13, %21;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %14, %21;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %15, %21;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %16, %21;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "mul.wide.u32 w, %17, %21;\n\t"
            "mov.b64 {%6, hi6}, w;\n\t"
            "mul.wide.u32 w, %18, %21;\n\t"
            "mov.b64 {%7, hi7}, w;\n\t"
            "mul.wide.u32 w, %19, %21;\n\t"
            "mov.b64 {%8, hi8}, w;\n\t"
            "mul.wide.u32 w, %20, %21;\n\t"
            "mov.b64 {%9, hi9}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.cc.u32 %6, %6, hi5;\n\t"
            "addc.cc.u32 %7, %7, hi6;\n\t"
            "addc.cc.u32 %8, %8, hi7;\n\t"
            "addc.cc.u32 %9, %9, hi8;\n\t"
            "addc.u32 %10, hi9, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6]), "=&r"(Q[7]), "=&r"(Q[8]), "=&r"(Q[9]), "=&r"(Q[10])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(y));
    }
};

template <>
struct MulWordOop<11> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<11>;\n\t"
            "mul.wide.u32 w, %12, %23;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %13, %23;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %14, %23;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %15, %23;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %16, %23;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %17, %23;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "mul.wide.u32 w, %18, %23;\n\t"
            "mov.b64 {%6, hi6}, w;\n\t"
            "mul.wide.u32 w, %19, %23;\n\t"
            "mov.b64 {%7, hi7}, w;\n\t"
            "mul.wide.u32 w, %20, %23;\n\t"
            "mov.b64 {%8, hi8}, w;\n\t"
            "mul.wide.u32 w, %21, %23;\n\t"
            "mov.b64 {%9, hi9}, w;\n\t"
            "mul.wide.u32 w, %22, %23;\n\t"
            "mov.b64 {%10, hi10}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.cc.u32 %6, %6, hi5;\n\t"
            "addc.cc.u32 %7, %7, hi6;\n\t"
            "addc.cc.u32 %8, %8, hi7;\n\t"
            "addc.cc.u32 %9, %9, hi8;\n\t"
            "addc.cc.u32 %10, %10, hi9;\n\t"
            "addc.u32 %11, hi10, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6]), "=&r"(Q[7]), "=&r"(Q[8]), "=&r"(Q[9]), "=&r"(Q[10]), "=&r"(Q[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(P[10]), "r"(y));
    }
};

template <>
struct MulWordOop<12> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<12>;\n\t"
            "mul.wide.u32 w, %13, %25;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %14, %25;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %15, %25;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %16, %25;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %17, %25;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %18, %25;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "mul.wide.u32 w, %19, %25;\n\t"
            "mov.b64 {%6, hi6}, w;\n\t"
            "mul.wide.u32 w, %20, %25;\n\t"
            "mov.b64 {%7, hi7}, w;\n\t"
            "mul.wide.u32 w, %21, %25;\n\t"
            "mov.b64 {%8, hi8}, w;\n\t"
            "mul.wide.u32 w, %22, %25;\n\t"
            "mov.b64 {%9, hi9}, w;\n\t"
            "mul.wide.u32 w, %23, %25;\n\t"
            "mov.b64 {%10, hi10}, w;\n\t"
            "mul.wide.u32 w, %24, %25;\n\t"
            "mov.b64 {%11, hi11}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.cc.u32 %6, %6, hi5;\n\t"
            "addc.cc.u32 %7, %7, hi6;\n\t"
            "addc.cc.u32 %8, %8, hi7;\n\t"
            "addc.cc.u32 %9, %9, hi8;\n\t"
            "addc.cc.u32 %10, %10, hi9;\n\t"
            "addc.cc.u32 %11, %11, hi10;\n\t"
            "addc.u32 %12, hi11, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6]), "=&r"(Q[7]), "=&r"(Q[8]), "=&r"(Q[9]), "=&r"(Q[10]), "=&r"(Q[11]), "=&r"(Q[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(P[10]), "r"(P[11]), "r"(y));
    }
};

template <>
struct MulWordOop<13> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<13>;\n\t"
            "mul.wide.u32 w, %14, %27;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %15, %27;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %16, %27;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %17, %27;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %18, %27;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %19, %27;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "mul.wide.u32 w, %20, %27;\n\t"
            "mov.b64 {%6, hi6}, w;\n\t"
            "mul.wide.u32 w, %21, %27;\n\t"
            "mov.b64 {%7, hi7}, w;\n\t"
            "mul.wide.u32 w, %22, %27;\n\t"
            "mov.b64 {%8, hi8}, w;\n\t"
            "mul.wide.u32 w, %23, %27;\n\t"
            "mov.b64 {%9, hi9}, w;\n\t"
            "mul.wide.u32 w, %24, %27;\n\t"
            "mov.b64 {%10, hi10}, w;\n\t"
            "mul.wide.u32 w, %25, %27;\n\t"
            "mov.b64 {%11, hi11}, w;\n\t"
            "mul.wide.u32 w, %26, %27;\n\t"
            "mov.b64 {%12, hi12}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.cc.u32 %6, %6, hi5;\n\t"
            "addc.cc.u32 %7, %7, hi6;\n\t"
            "addc.cc.u32 %8, %8, hi7;\n\t"
            "addc.cc.u32 %9, %9, hi8;\n\t"
            "addc.cc.u32 %10, %10, hi9;\n\t"
            "addc.cc.u32 %11, %11, hi10;\n\t"
            "addc.cc.u32 %12, %12, hi11;\n\t"
            "addc.u32 %13, hi12, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6]), "=&r"(Q[7]), "=&r"(Q[8]), "=&r"(Q[9]), "=&r"(Q[10]), "=&r"(Q[11]), "=&r"(Q[12]), "=&r"(Q[13])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(P[10]), "r"(P[11]), "r"(P[12]), "r"(y));
    }
};

template <>
struct MulWordOop<14> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<14>;\n\t"
            "mul.wide.u32 w, %15, %29;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %16, %29;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %17, %29;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %18, %29;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %19, %29;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %20, %29;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "mul.wide.u32 w, %21, %29;\n\t"
            "mov.b64 {%6, hi6}, w;\n\t"
            "mul.wide.u32 w, %22, %29;\n\t"
            "mov.b64 {%7, hi7}, w;\n\t"
            "mul.wide.u32 w, %23, %29;\n\t"
            "mov.b64 {%8, hi8}, w;\n\t"
            "mul.wide.u32 w, %24, %29;\n\t"
            "mov.b64 {%9, hi9}, w;\n\t"
            "mul.wide.u32 w, %25, %29;\n\t"
            "mov.b64 {%10, hi10}, w;\n\t"
            "mul.wide.u32 w, %26, %29;\n\t"
            "mov.b64 {%11, hi11}, w;\n\t"
            "mul.wide.u32 w, %27, %29;\n\t"
            "mov.b64 {%12, hi12}, w;\n\t"
            "mul.wide.u32 w, %28, %29;\n\t"
            "mov.b64 {%13, hi13}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.cc.u32 %6, %6, hi5;\n\t"
            "addc.cc.u32 %7, %7, hi6;\n\t"
            "addc.cc.u32 %8, %8, hi7;\n\t"
            "addc.cc.u32 %9, %9, hi8;\n\t"
            "addc.cc.u32 %10, %10, hi9;\n\t"
            "addc.cc.u32 %11, %11, hi10;\n\t"
            "addc.cc.u32 %12, %12, hi11;\n\t"
            "addc.cc.u32 %13, %13, hi12;\n\t"
            "addc.u32 %14, hi13, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6]), "=&r"(Q[7]), "=&r"(Q[8]), "=&r"(Q[9]), "=&r"(Q[10]), "=&r"(Q[11]), "=&r"(Q[12]), "=&r"(Q[13]), "=&r"(Q[14])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(P[10]), "r"(P[11]), "r"(P[12]), "r"(P[13]), "r"(y));
    }
};

template <>
struct MulWordOop<15> {
    static __device__ __forceinline__ void apply(const uint32_t *P, uint32_t *Q, uint32_t y) {
        asm("{\n\t"
            ".reg .u64 w;\n\t"
            ".reg .u32 hi<15>;\n\t"
            "mul.wide.u32 w, %16, %31;\n\t"
            "mov.b64 {%0, hi0}, w;\n\t"
            "mul.wide.u32 w, %17, %31;\n\t"
            "mov.b64 {%1, hi1}, w;\n\t"
            "mul.wide.u32 w, %18, %31;\n\t"
            "mov.b64 {%2, hi2}, w;\n\t"
            "mul.wide.u32 w, %19, %31;\n\t"
            "mov.b64 {%3, hi3}, w;\n\t"
            "mul.wide.u32 w, %20, %31;\n\t"
            "mov.b64 {%4, hi4}, w;\n\t"
            "mul.wide.u32 w, %21, %31;\n\t"
            "mov.b64 {%5, hi5}, w;\n\t"
            "mul.wide.u32 w, %22, %31;\n\t"
            "mov.b64 {%6, hi6}, w;\n\t"
            "mul.wide.u32 w, %23, %31;\n\t"
            "mov.b64 {%7, hi7}, w;\n\t"
            "mul.wide.u32 w, %24, %31;\n\t"
            "mov.b64 {%8, hi8}, w;\n\t"
            "mul.wide.u32 w, %25, %31;\n\t"
            "mov.b64 {%9, hi9}, w;\n\t"
            "mul.wide.u32 w, %26, %31;\n\t"
            "mov.b64 {%10, hi10}, w;\n\t"
            "mul.wide.u32 w, %27, %31;\n\t"
            "mov.b64 {%11, hi11}, w;\n\t"
            "mul.wide.u32 w, %28, %31;\n\t"
            "mov.b64 {%12, hi12}, w;\n\t"
            "mul.wide.u32 w, %29, %31;\n\t"
            "mov.b64 {%13, hi13}, w;\n\t"
            "mul.wide.u32 w, %30, %31;\n\t"
            "mov.b64 {%14, hi14}, w;\n\t"
            "add.cc.u32 %1, %1, hi0;\n\t"
            "addc.cc.u32 %2, %2, hi1;\n\t"
            "addc.cc.u32 %3, %3, hi2;\n\t"
            "addc.cc.u32 %4, %4, hi3;\n\t"
            "addc.cc.u32 %5, %5, hi4;\n\t"
            "addc.cc.u32 %6, %6, hi5;\n\t"
            "addc.cc.u32 %7, %7, hi6;\n\t"
            "addc.cc.u32 %8, %8, hi7;\n\t"
            "addc.cc.u32 %9, %9, hi8;\n\t"
            "addc.cc.u32 %10, %10, hi9;\n\t"
            "addc.cc.u32 %11, %11, hi10;\n\t"
            "addc.cc.u32 %12, %12, hi11;\n\t"
            "addc.cc.u32 %13, %13, hi12;\n\t"
            "addc.cc.u32 %14, %14, hi13;\n\t"
            "addc.u32 %15, hi14, 0;\n\t"
            "}"
            : "=&r"(Q[0]), "=&r"(Q[1]), "=&r"(Q[2]), "=&r"(Q[3]), "=&r"(Q[4]), "=&r"(Q[5]), "=&r"(Q[6]), "=&r"(Q[7]), "=&r"(Q[8]), "=&r"(Q[9]), "=&r"(Q[10]), "=&r"(Q[11]), "=&r"(Q[12]), "=&r"(Q[13]), "=&r"(Q[14]), "=&r"(Q[15])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(P[10]), "r"(P[11]), "r"(P[12]), "r"(P[13]), "r"(P[14]), "r"(y));
    }
};

}  // namespace pg
