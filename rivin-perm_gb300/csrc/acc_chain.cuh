// Signed accumulation of an exact Glynn term into a multi-word accumulator:
//   acc (NL words, two's complement) += (-1)^neg * P (NG unsigned words),
// as one PTX carry chain: CF := neg (add.cc m, m with m = 0 or ~0), then
// acc_l += P_l ^ m (+ carry) for l < NG and acc_l += m for the sign words.
// Generated for NL <= 13; larger shapes use the portable loop below.
#pragma once
#include <stdint.h>

namespace pg {

template <int NL, int NG>
struct AccChain {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        uint32_t cy = m & 1u;
#pragma unroll
        for (int l = 0; l < NL; l++) {
            const uint32_t w = (l < NG ? P[l] : 0u) ^ m;
            const uint64_t t = (uint64_t)acc[l] + w + cy;
            acc[l] = (uint32_t)t;
            cy = (uint32_t)(t >> 32);
        }
    }
};

template <>
struct AccChain<2, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %3, %3;\n\t"
            "xor.b32 t, %2, %3;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.u32 %1, %1, %3;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<3, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %4, %4;\n\t"
            "xor.b32 t, %3, %4;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %4;\n\t"
            "addc.u32 %2, %2, %4;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<3, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %5, %5;\n\t"
            "xor.b32 t, %3, %5;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %4, %5;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.u32 %2, %2, %5;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<4, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %5, %5;\n\t"
            "xor.b32 t, %4, %5;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %5;\n\t"
            "addc.cc.u32 %2, %2, %5;\n\t"
            "addc.u32 %3, %3, %5;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<4, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %6, %6;\n\t"
            "xor.b32 t, %4, %6;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %5, %6;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %6;\n\t"
            "addc.u32 %3, %3, %6;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<4, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %7, %7;\n\t"
            "xor.b32 t, %4, %7;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %5, %7;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %6, %7;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.u32 %3, %3, %7;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<5, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %6, %6;\n\t"
            "xor.b32 t, %5, %6;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %6;\n\t"
            "addc.cc.u32 %2, %2, %6;\n\t"
            "addc.cc.u32 %3, %3, %6;\n\t"
            "addc.u32 %4, %4, %6;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<5, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %7, %7;\n\t"
            "xor.b32 t, %5, %7;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %6, %7;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %7;\n\t"
            "addc.cc.u32 %3, %3, %7;\n\t"
            "addc.u32 %4, %4, %7;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<5, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %8, %8;\n\t"
            "xor.b32 t, %5, %8;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %6, %8;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %7, %8;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.cc.u32 %3, %3, %8;\n\t"
            "addc.u32 %4, %4, %8;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<5, 4> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %9, %9;\n\t"
            "xor.b32 t, %5, %9;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %6, %9;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %7, %9;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %8, %9;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "addc.u32 %4, %4, %9;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(m));
    }
};

template <>
struct AccChain<6, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %7, %7;\n\t"
            "xor.b32 t, %6, %7;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %7;\n\t"
            "addc.cc.u32 %2, %2, %7;\n\t"
            "addc.cc.u32 %3, %3, %7;\n\t"
            "addc.cc.u32 %4, %4, %7;\n\t"
            "addc.u32 %5, %5, %7;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<6, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %8, %8;\n\t"
            "xor.b32 t, %6, %8;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %7, %8;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %8;\n\t"
            "addc.cc.u32 %3, %3, %8;\n\t"
            "addc.cc.u32 %4, %4, %8;\n\t"
            "addc.u32 %5, %5, %8;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<6, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %9, %9;\n\t"
            "xor.b32 t, %6, %9;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %7, %9;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %8, %9;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.cc.u32 %3, %3, %9;\n\t"
            "addc.cc.u32 %4, %4, %9;\n\t"
            "addc.u32 %5, %5, %9;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<6, 4> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %10, %10;\n\t"
            "xor.b32 t, %6, %10;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %7, %10;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %8, %10;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %9, %10;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "addc.cc.u32 %4, %4, %10;\n\t"
            "addc.u32 %5, %5, %10;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(m));
    }
};

template <>
struct AccChain<6, 5> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %11, %11;\n\t"
            "xor.b32 t, %6, %11;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %7, %11;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %8, %11;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %9, %11;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %10, %11;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "addc.u32 %5, %5, %11;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(m));
    }
};

template <>
struct AccChain<7, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %8, %8;\n\t"
            "xor.b32 t, %7, %8;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %8;\n\t"
            "addc.cc.u32 %2, %2, %8;\n\t"
            "addc.cc.u32 %3, %3, %8;\n\t"
            "addc.cc.u32 %4, %4, %8;\n\t"
            "addc.cc.u32 %5, %5, %8;\n\t"
            "addc.u32 %6, %6, %8;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<7, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %9, %9;\n\t"
            "xor.b32 t, %7, %9;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %8, %9;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %9;\n\t"
            "addc.cc.u32 %3, %3, %9;\n\t"
            "addc.cc.u32 %4, %4, %9;\n\t"
            "addc.cc.u32 %5, %5, %9;\n\t"
            "addc.u32 %6, %6, %9;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<7, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %10, %10;\n\t"
            "xor.b32 t, %7, %10;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %8, %10;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %9, %10;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.cc.u32 %3, %3, %10;\n\t"
            "addc.cc.u32 %4, %4, %10;\n\t"
            "addc.cc.u32 %5, %5, %10;\n\t"
            "addc.u32 %6, %6, %10;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<7, 4> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %11, %11;\n\t"
            "xor.b32 t, %7, %11;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %8, %11;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %9, %11;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %10, %11;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "addc.cc.u32 %4, %4, %11;\n\t"
            "addc.cc.u32 %5, %5, %11;\n\t"
            "addc.u32 %6, %6, %11;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(m));
    }
};

template <>
struct AccChain<7, 5> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %12, %12;\n\t"
            "xor.b32 t, %7, %12;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %8, %12;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %9, %12;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %10, %12;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %11, %12;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "addc.cc.u32 %5, %5, %12;\n\t"
            "addc.u32 %6, %6, %12;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(m));
    }
};

template <>
struct AccChain<7, 6> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %13, %13;\n\t"
            "xor.b32 t, %7, %13;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %8, %13;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %9, %13;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %10, %13;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %11, %13;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %12, %13;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "addc.u32 %6, %6, %13;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(m));
    }
};

template <>
struct AccChain<8, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %9, %9;\n\t"
            "xor.b32 t, %8, %9;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %9;\n\t"
            "addc.cc.u32 %2, %2, %9;\n\t"
            "addc.cc.u32 %3, %3, %9;\n\t"
            "addc.cc.u32 %4, %4, %9;\n\t"
            "addc.cc.u32 %5, %5, %9;\n\t"
            "addc.cc.u32 %6, %6, %9;\n\t"
            "addc.u32 %7, %7, %9;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<8, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %10, %10;\n\t"
            "xor.b32 t, %8, %10;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %9, %10;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %10;\n\t"
            "addc.cc.u32 %3, %3, %10;\n\t"
            "addc.cc.u32 %4, %4, %10;\n\t"
            "addc.cc.u32 %5, %5, %10;\n\t"
            "addc.cc.u32 %6, %6, %10;\n\t"
            "addc.u32 %7, %7, %10;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<8, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %11, %11;\n\t"
            "xor.b32 t, %8, %11;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %9, %11;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %10, %11;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.cc.u32 %3, %3, %11;\n\t"
            "addc.cc.u32 %4, %4, %11;\n\t"
            "addc.cc.u32 %5, %5, %11;\n\t"
            "addc.cc.u32 %6, %6, %11;\n\t"
            "addc.u32 %7, %7, %11;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<8, 4> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %12, %12;\n\t"
            "xor.b32 t, %8, %12;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %9, %12;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %10, %12;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %11, %12;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "addc.cc.u32 %4, %4, %12;\n\t"
            "addc.cc.u32 %5, %5, %12;\n\t"
            "addc.cc.u32 %6, %6, %12;\n\t"
            "addc.u32 %7, %7, %12;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(m));
    }
};

template <>
struct AccChain<8, 5> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %13, %13;\n\t"
            "xor.b32 t, %8, %13;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %9, %13;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %10, %13;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %11, %13;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %12, %13;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "addc.cc.u32 %5, %5, %13;\n\t"
            "addc.cc.u32 %6, %6, %13;\n\t"
            "addc.u32 %7, %7, %13;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(m));
    }
};

template <>
struct AccChain<8, 6> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %14, %14;\n\t"
            "xor.b32 t, %8, %14;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %9, %14;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %10, %14;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %11, %14;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %12, %14;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %13, %14;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "addc.cc.u32 %6, %6, %14;\n\t"
            "addc.u32 %7, %7, %14;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(m));
    }
};

template <>
struct AccChain<8, 7> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %15, %15;\n\t"
            "xor.b32 t, %8, %15;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %9, %15;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %10, %15;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %11, %15;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %12, %15;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %13, %15;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %14, %15;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "addc.u32 %7, %7, %15;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(m));
    }
};

template <>
struct AccChain<9, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %10, %10;\n\t"
            "xor.b32 t, %9, %10;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %10;\n\t"
            "addc.cc.u32 %2, %2, %10;\n\t"
            "addc.cc.u32 %3, %3, %10;\n\t"
            "addc.cc.u32 %4, %4, %10;\n\t"
            "addc.cc.u32 %5, %5, %10;\n\t"
            "addc.cc.u32 %6, %6, %10;\n\t"
            "addc.cc.u32 %7, %7, %10;\n\t"
            "addc.u32 %8, %8, %10;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<9, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %11, %11;\n\t"
            "xor.b32 t, %9, %11;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %10, %11;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %11;\n\t"
            "addc.cc.u32 %3, %3, %11;\n\t"
            "addc.cc.u32 %4, %4, %11;\n\t"
            "addc.cc.u32 %5, %5, %11;\n\t"
            "addc.cc.u32 %6, %6, %11;\n\t"
            "addc.cc.u32 %7, %7, %11;\n\t"
            "addc.u32 %8, %8, %11;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<9, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %12, %12;\n\t"
            "xor.b32 t, %9, %12;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %10, %12;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %11, %12;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.cc.u32 %3, %3, %12;\n\t"
            "addc.cc.u32 %4, %4, %12;\n\t"
            "addc.cc.u32 %5, %5, %12;\n\t"
            "addc.cc.u32 %6, %6, %12;\n\t"
            "addc.cc.u32 %7, %7, %12;\n\t"
            "addc.u32 %8, %8, %12;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<9, 4> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %13, %13;\n\t"
            "xor.b32 t, %9, %13;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %10, %13;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %11, %13;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %12, %13;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "addc.cc.u32 %4, %4, %13;\n\t"
            "addc.cc.u32 %5, %5, %13;\n\t"
            "addc.cc.u32 %6, %6, %13;\n\t"
            "addc.cc.u32 %7, %7, %13;\n\t"
            "addc.u32 %8, %8, %13;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(m));
    }
};

template <>
struct AccChain<9, 5> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %14, %14;\n\t"
            "xor.b32 t, %9, %14;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %10, %14;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %11, %14;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %12, %14;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %13, %14;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "addc.cc.u32 %5, %5, %14;\n\t"
            "addc.cc.u32 %6, %6, %14;\n\t"
            "addc.cc.u32 %7, %7, %14;\n\t"
            "addc.u32 %8, %8, %14;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(m));
    }
};

template <>
struct AccChain<9, 6> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %15, %15;\n\t"
            "xor.b32 t, %9, %15;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %10, %15;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %11, %15;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %12, %15;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %13, %15;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %14, %15;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "addc.cc.u32 %6, %6, %15;\n\t"
            "addc.cc.u32 %7, %7, %15;\n\t"
            "addc.u32 %8, %8, %15;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(m));
    }
};

template <>
struct AccChain<9, 7> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %16, %16;\n\t"
            "xor.b32 t, %9, %16;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %10, %16;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %11, %16;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %12, %16;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %13, %16;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %14, %16;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %15, %16;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "addc.cc.u32 %7, %7, %16;\n\t"
            "addc.u32 %8, %8, %16;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(m));
    }
};

template <>
struct AccChain<9, 8> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %17, %17;\n\t"
            "xor.b32 t, %9, %17;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %10, %17;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %11, %17;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %12, %17;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %13, %17;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %14, %17;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %15, %17;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %16, %17;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "addc.u32 %8, %8, %17;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(m));
    }
};

template <>
struct AccChain<10, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %11, %11;\n\t"
            "xor.b32 t, %10, %11;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %11;\n\t"
            "addc.cc.u32 %2, %2, %11;\n\t"
            "addc.cc.u32 %3, %3, %11;\n\t"
            "addc.cc.u32 %4, %4, %11;\n\t"
            "addc.cc.u32 %5, %5, %11;\n\t"
            "addc.cc.u32 %6, %6, %11;\n\t"
            "addc.cc.u32 %7, %7, %11;\n\t"
            "addc.cc.u32 %8, %8, %11;\n\t"
            "addc.u32 %9, %9, %11;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<10, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %12, %12;\n\t"
            "xor.b32 t, %10, %12;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %11, %12;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %12;\n\t"
            "addc.cc.u32 %3, %3, %12;\n\t"
            "addc.cc.u32 %4, %4, %12;\n\t"
            "addc.cc.u32 %5, %5, %12;\n\t"
            "addc.cc.u32 %6, %6, %12;\n\t"
            "addc.cc.u32 %7, %7, %12;\n\t"
            "addc.cc.u32 %8, %8, %12;\n\t"
            "addc.u32 %9, %9, %12;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<10, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %13, %13;\n\t"
            "xor.b32 t, %10, %13;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %11, %13;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %12, %13;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.cc.u32 %3, %3, %13;\n\t"
            "addc.cc.u32 %4, %4, %13;\n\t"
            "addc.cc.u32 %5, %5, %13;\n\t"
            "addc.cc.u32 %6, %6, %13;\n\t"
            "addc.cc.u32 %7, %7, %13;\n\t"
            "addc.cc.u32 %8, %8, %13;\n\t"
            "addc.u32 %9, %9, %13;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<10, 4> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %14, %14;\n\t"
            "xor.b32 t, %10, %14;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %11, %14;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %12, %14;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %13, %14;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "addc.cc.u32 %4, %4, %14;\n\t"
            "addc.cc.u32 %5, %5, %14;\n\t"
            "addc.cc.u32 %6, %6, %14;\n\t"
            "addc.cc.u32 %7, %7, %14;\n\t"
            "addc.cc.u32 %8, %8, %14;\n\t"
            "addc.u32 %9, %9, %14;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(m));
    }
};

template <>
struct AccChain<10, 5> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %15, %15;\n\t"
            "xor.b32 t, %10, %15;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %11, %15;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %12, %15;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %13, %15;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %14, %15;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "addc.cc.u32 %5, %5, %15;\n\t"
            "addc.cc.u32 %6, %6, %15;\n\t"
            "addc.cc.u32 %7, %7, %15;\n\t"
            "addc.cc.u32 %8, %8, %15;\n\t"
            "addc.u32 %9, %9, %15;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(m));
    }
};

template <>
struct AccChain<10, 6> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %16, %16;\n\t"
            "xor.b32 t, %10, %16;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %11, %16;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %12, %16;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %13, %16;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %14, %16;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %15, %16;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "addc.cc.u32 %6, %6, %16;\n\t"
            "addc.cc.u32 %7, %7, %16;\n\t"
            "addc.cc.u32 %8, %8, %16;\n\t"
            "addc.u32 %9, %9, %16;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(m));
    }
};

template <>
struct AccChain<10, 7> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %17, %17;\n\t"
            "xor.b32 t, %10, %17;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %11, %17;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %12, %17;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %13, %17;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %14, %17;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %15, %17;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %16, %17;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "addc.cc.u32 %7, %7, %17;\n\t"
            "addc.cc.u32 %8, %8, %17;\n\t"
            "addc.u32 %9, %9, %17;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(m));
    }
};

template <>
struct AccChain<10, 8> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %18, %18;\n\t"
            "xor.b32 t, %10, %18;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %11, %18;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %12, %18;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %13, %18;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %14, %18;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %15, %18;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %16, %18;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %17, %18;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "addc.cc.u32 %8, %8, %18;\n\t"
            "addc.u32 %9, %9, %18;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(m));
    }
};

template <>
struct AccChain<10, 9> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %19, %19;\n\t"
            "xor.b32 t, %10, %19;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %11, %19;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %12, %19;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %13, %19;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %14, %19;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %15, %19;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %16, %19;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %17, %19;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %18, %19;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "addc.u32 %9, %9, %19;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(m));
    }
};

template <>
struct AccChain<11, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %12, %12;\n\t"
            "xor.b32 t, %11, %12;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %12;\n\t"
            "addc.cc.u32 %2, %2, %12;\n\t"
            "addc.cc.u32 %3, %3, %12;\n\t"
            "addc.cc.u32 %4, %4, %12;\n\t"
            "addc.cc.u32 %5, %5, %12;\n\t"
            "addc.cc.u32 %6, %6, %12;\n\t"
            "addc.cc.u32 %7, %7, %12;\n\t"
            "addc.cc.u32 %8, %8, %12;\n\t"
            "addc.cc.u32 %9, %9, %12;\n\t"
            "addc.u32 %10, %10, %12;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<11, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %13, %13;\n\t"
            "xor.b32 t, %11, %13;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %12, %13;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %13;\n\t"
            "addc.cc.u32 %3, %3, %13;\n\t"
            "addc.cc.u32 %4, %4, %13;\n\t"
            "addc.cc.u32 %5, %5, %13;\n\t"
            "addc.cc.u32 %6, %6, %13;\n\t"
            "addc.cc.u32 %7, %7, %13;\n\t"
            "addc.cc.u32 %8, %8, %13;\n\t"
            "addc.cc.u32 %9, %9, %13;\n\t"
            "addc.u32 %10, %10, %13;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<11, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %14, %14;\n\t"
            "xor.b32 t, %11, %14;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %12, %14;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %13, %14;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.cc.u32 %3, %3, %14;\n\t"
            "addc.cc.u32 %4, %4, %14;\n\t"
            "addc.cc.u32 %5, %5, %14;\n\t"
            "addc.cc.u32 %6, %6, %14;\n\t"
            "addc.cc.u32 %7, %7, %14;\n\t"
            "addc.cc.u32 %8, %8, %14;\n\t"
            "addc.cc.u32 %9, %9, %14;\n\t"
            "addc.u32 %10, %10, %14;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<11, 4> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %15, %15;\n\t"
            "xor.b32 t, %11, %15;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %12, %15;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %13, %15;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %14, %15;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "addc.cc.u32 %4, %4, %15;\n\t"
            "addc.cc.u32 %5, %5, %15;\n\t"
            "addc.cc.u32 %6, %6, %15;\n\t"
            "addc.cc.u32 %7, %7, %15;\n\t"
            "addc.cc.u32 %8, %8, %15;\n\t"
            "addc.cc.u32 %9, %9, %15;\n\t"
            "addc.u32 %10, %10, %15;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(m));
    }
};

template <>
struct AccChain<11, 5> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %16, %16;\n\t"
            "xor.b32 t, %11, %16;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %12, %16;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %13, %16;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %14, %16;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %15, %16;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "addc.cc.u32 %5, %5, %16;\n\t"
            "addc.cc.u32 %6, %6, %16;\n\t"
            "addc.cc.u32 %7, %7, %16;\n\t"
            "addc.cc.u32 %8, %8, %16;\n\t"
            "addc.cc.u32 %9, %9, %16;\n\t"
            "addc.u32 %10, %10, %16;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(m));
    }
};

template <>
struct AccChain<11, 6> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %17, %17;\n\t"
            "xor.b32 t, %11, %17;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %12, %17;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %13, %17;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %14, %17;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %15, %17;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %16, %17;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "addc.cc.u32 %6, %6, %17;\n\t"
            "addc.cc.u32 %7, %7, %17;\n\t"
            "addc.cc.u32 %8, %8, %17;\n\t"
            "addc.cc.u32 %9, %9, %17;\n\t"
            "addc.u32 %10, %10, %17;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(m));
    }
};

template <>
struct AccChain<11, 7> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %18, %18;\n\t"
            "xor.b32 t, %11, %18;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %12, %18;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %13, %18;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %14, %18;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %15, %18;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %16, %18;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %17, %18;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "addc.cc.u32 %7, %7, %18;\n\t"
            "addc.cc.u32 %8, %8, %18;\n\t"
            "addc.cc.u32 %9, %9, %18;\n\t"
            "addc.u32 %10, %10, %18;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(m));
    }
};

template <>
struct AccChain<11, 8> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %19, %19;\n\t"
            "xor.b32 t, %11, %19;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %12, %19;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %13, %19;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %14, %19;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %15, %19;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %16, %19;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %17, %19;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %18, %19;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "addc.cc.u32 %8, %8, %19;\n\t"
            "addc.cc.u32 %9, %9, %19;\n\t"
            "addc.u32 %10, %10, %19;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(m));
    }
};

template <>
struct AccChain<11, 9> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %20, %20;\n\t"
            "xor.b32 t, %11, %20;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %12, %20;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %13, %20;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %14, %20;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %15, %20;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %16, %20;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %17, %20;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %18, %20;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %19, %20;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "addc.cc.u32 %9, %9, %20;\n\t"
            "addc.u32 %10, %10, %20;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(m));
    }
};

template <>
struct AccChain<11, 10> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %21, %21;\n\t"
            "xor.b32 t, %11, %21;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %12, %21;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %13, %21;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %14, %21;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %15, %21;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %16, %21;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %17, %21;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %18, %21;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %19, %21;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "xor.b32 t, %20, %21;\n\t"
            "addc.cc.u32 %9, %9, t;\n\t"
            "addc.u32 %10, %10, %21;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(m));
    }
};

template <>
struct AccChain<12, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %13, %13;\n\t"
            "xor.b32 t, %12, %13;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %13;\n\t"
            "addc.cc.u32 %3, %3, %13;\n\t"
            "addc.cc.u32 %4, %4, %13;\n\t"
            "addc.cc.u32 %5, %5, %13;\n\t"
            "addc.cc.u32 %6, %6, %13;\n\t"
            "addc.cc.u32 %7, %7, %13;\n\t"
            "addc.cc.u32 %8, %8, %13;\n\t"
            "addc.cc.u32 %9, %9, %13;\n\t"
            "addc.cc.u32 %10, %10, %13;\n\t"
            "addc.u32 %11, %11, %13;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<12, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %14, %14;\n\t"
            "xor.b32 t, %12, %14;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %14;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %14;\n\t"
            "addc.cc.u32 %4, %4, %14;\n\t"
            "addc.cc.u32 %5, %5, %14;\n\t"
            "addc.cc.u32 %6, %6, %14;\n\t"
            "addc.cc.u32 %7, %7, %14;\n\t"
            "addc.cc.u32 %8, %8, %14;\n\t"
            "addc.cc.u32 %9, %9, %14;\n\t"
            "addc.cc.u32 %10, %10, %14;\n\t"
            "addc.u32 %11, %11, %14;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<12, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %15, %15;\n\t"
            "xor.b32 t, %12, %15;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %15;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %14, %15;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %15;\n\t"
            "addc.cc.u32 %5, %5, %15;\n\t"
            "addc.cc.u32 %6, %6, %15;\n\t"
            "addc.cc.u32 %7, %7, %15;\n\t"
            "addc.cc.u32 %8, %8, %15;\n\t"
            "addc.cc.u32 %9, %9, %15;\n\t"
            "addc.cc.u32 %10, %10, %15;\n\t"
            "addc.u32 %11, %11, %15;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<12, 4> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %16, %16;\n\t"
            "xor.b32 t, %12, %16;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %16;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %14, %16;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %15, %16;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %16;\n\t"
            "addc.cc.u32 %6, %6, %16;\n\t"
            "addc.cc.u32 %7, %7, %16;\n\t"
            "addc.cc.u32 %8, %8, %16;\n\t"
            "addc.cc.u32 %9, %9, %16;\n\t"
            "addc.cc.u32 %10, %10, %16;\n\t"
            "addc.u32 %11, %11, %16;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(m));
    }
};

template <>
struct AccChain<12, 5> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %17, %17;\n\t"
            "xor.b32 t, %12, %17;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %17;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %14, %17;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %15, %17;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %16, %17;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %17;\n\t"
            "addc.cc.u32 %7, %7, %17;\n\t"
            "addc.cc.u32 %8, %8, %17;\n\t"
            "addc.cc.u32 %9, %9, %17;\n\t"
            "addc.cc.u32 %10, %10, %17;\n\t"
            "addc.u32 %11, %11, %17;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(m));
    }
};

template <>
struct AccChain<12, 6> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %18, %18;\n\t"
            "xor.b32 t, %12, %18;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %18;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %14, %18;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %15, %18;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %16, %18;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %17, %18;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %18;\n\t"
            "addc.cc.u32 %8, %8, %18;\n\t"
            "addc.cc.u32 %9, %9, %18;\n\t"
            "addc.cc.u32 %10, %10, %18;\n\t"
            "addc.u32 %11, %11, %18;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(m));
    }
};

template <>
struct AccChain<12, 7> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %19, %19;\n\t"
            "xor.b32 t, %12, %19;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %19;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %14, %19;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %15, %19;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %16, %19;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %17, %19;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %18, %19;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %19;\n\t"
            "addc.cc.u32 %9, %9, %19;\n\t"
            "addc.cc.u32 %10, %10, %19;\n\t"
            "addc.u32 %11, %11, %19;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(m));
    }
};

template <>
struct AccChain<12, 8> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %20, %20;\n\t"
            "xor.b32 t, %12, %20;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %20;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %14, %20;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %15, %20;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %16, %20;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %17, %20;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %18, %20;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %19, %20;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %20;\n\t"
            "addc.cc.u32 %10, %10, %20;\n\t"
            "addc.u32 %11, %11, %20;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(m));
    }
};

template <>
struct AccChain<12, 9> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %21, %21;\n\t"
            "xor.b32 t, %12, %21;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %21;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %14, %21;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %15, %21;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %16, %21;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %17, %21;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %18, %21;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %19, %21;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %20, %21;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %21;\n\t"
            "addc.u32 %11, %11, %21;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(m));
    }
};

template <>
struct AccChain<12, 10> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %22, %22;\n\t"
            "xor.b32 t, %12, %22;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %22;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %14, %22;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %15, %22;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %16, %22;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %17, %22;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %18, %22;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %19, %22;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %20, %22;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "xor.b32 t, %21, %22;\n\t"
            "addc.cc.u32 %9, %9, t;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32 %11, %11, %22;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(m));
    }
};

template <>
struct AccChain<12, 11> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %23, %23;\n\t"
            "xor.b32 t, %12, %23;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %13, %23;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %14, %23;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %15, %23;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %16, %23;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %17, %23;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %18, %23;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %19, %23;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %20, %23;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "xor.b32 t, %21, %23;\n\t"
            "addc.cc.u32 %9, %9, t;\n\t"
            "xor.b32 t, %22, %23;\n\t"
            "addc.cc.u32 %10, %10, t;\n\t"
            "addc.u32 %11, %11, %23;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(P[10]), "r"(m));
    }
};

template <>
struct AccChain<13, 1> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %14, %14;\n\t"
            "xor.b32 t, %13, %14;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "addc.cc.u32 %1, %1, %14;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %14;\n\t"
            "addc.cc.u32 %4, %4, %14;\n\t"
            "addc.cc.u32 %5, %5, %14;\n\t"
            "addc.cc.u32 %6, %6, %14;\n\t"
            "addc.cc.u32 %7, %7, %14;\n\t"
            "addc.cc.u32 %8, %8, %14;\n\t"
            "addc.cc.u32 %9, %9, %14;\n\t"
            "addc.cc.u32 %10, %10, %14;\n\t"
            "addc.cc.u32 %11, %11, %14;\n\t"
            "addc.u32 %12, %12, %14;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(m));
    }
};

template <>
struct AccChain<13, 2> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %15, %15;\n\t"
            "xor.b32 t, %13, %15;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %15;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "addc.cc.u32 %2, %2, %15;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %15;\n\t"
            "addc.cc.u32 %5, %5, %15;\n\t"
            "addc.cc.u32 %6, %6, %15;\n\t"
            "addc.cc.u32 %7, %7, %15;\n\t"
            "addc.cc.u32 %8, %8, %15;\n\t"
            "addc.cc.u32 %9, %9, %15;\n\t"
            "addc.cc.u32 %10, %10, %15;\n\t"
            "addc.cc.u32 %11, %11, %15;\n\t"
            "addc.u32 %12, %12, %15;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(m));
    }
};

template <>
struct AccChain<13, 3> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %16, %16;\n\t"
            "xor.b32 t, %13, %16;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %16;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %16;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "addc.cc.u32 %3, %3, %16;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %16;\n\t"
            "addc.cc.u32 %6, %6, %16;\n\t"
            "addc.cc.u32 %7, %7, %16;\n\t"
            "addc.cc.u32 %8, %8, %16;\n\t"
            "addc.cc.u32 %9, %9, %16;\n\t"
            "addc.cc.u32 %10, %10, %16;\n\t"
            "addc.cc.u32 %11, %11, %16;\n\t"
            "addc.u32 %12, %12, %16;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(m));
    }
};

template <>
struct AccChain<13, 4> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %17, %17;\n\t"
            "xor.b32 t, %13, %17;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %17;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %17;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %16, %17;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "addc.cc.u32 %4, %4, %17;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %17;\n\t"
            "addc.cc.u32 %7, %7, %17;\n\t"
            "addc.cc.u32 %8, %8, %17;\n\t"
            "addc.cc.u32 %9, %9, %17;\n\t"
            "addc.cc.u32 %10, %10, %17;\n\t"
            "addc.cc.u32 %11, %11, %17;\n\t"
            "addc.u32 %12, %12, %17;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(m));
    }
};

template <>
struct AccChain<13, 5> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %18, %18;\n\t"
            "xor.b32 t, %13, %18;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %18;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %18;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %16, %18;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %17, %18;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "addc.cc.u32 %5, %5, %18;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %18;\n\t"
            "addc.cc.u32 %8, %8, %18;\n\t"
            "addc.cc.u32 %9, %9, %18;\n\t"
            "addc.cc.u32 %10, %10, %18;\n\t"
            "addc.cc.u32 %11, %11, %18;\n\t"
            "addc.u32 %12, %12, %18;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(m));
    }
};

template <>
struct AccChain<13, 6> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %19, %19;\n\t"
            "xor.b32 t, %13, %19;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %19;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %19;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %16, %19;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %17, %19;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %18, %19;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "addc.cc.u32 %6, %6, %19;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %19;\n\t"
            "addc.cc.u32 %9, %9, %19;\n\t"
            "addc.cc.u32 %10, %10, %19;\n\t"
            "addc.cc.u32 %11, %11, %19;\n\t"
            "addc.u32 %12, %12, %19;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(m));
    }
};

template <>
struct AccChain<13, 7> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %20, %20;\n\t"
            "xor.b32 t, %13, %20;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %20;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %20;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %16, %20;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %17, %20;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %18, %20;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %19, %20;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "addc.cc.u32 %7, %7, %20;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %20;\n\t"
            "addc.cc.u32 %10, %10, %20;\n\t"
            "addc.cc.u32 %11, %11, %20;\n\t"
            "addc.u32 %12, %12, %20;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(m));
    }
};

template <>
struct AccChain<13, 8> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %21, %21;\n\t"
            "xor.b32 t, %13, %21;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %21;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %21;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %16, %21;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %17, %21;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %18, %21;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %19, %21;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %20, %21;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "addc.cc.u32 %8, %8, %21;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %21;\n\t"
            "addc.cc.u32 %11, %11, %21;\n\t"
            "addc.u32 %12, %12, %21;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(m));
    }
};

template <>
struct AccChain<13, 9> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %22, %22;\n\t"
            "xor.b32 t, %13, %22;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %22;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %22;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %16, %22;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %17, %22;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %18, %22;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %19, %22;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %20, %22;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %21, %22;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "addc.cc.u32 %9, %9, %22;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.cc.u32 %11, %11, %22;\n\t"
            "addc.u32 %12, %12, %22;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(m));
    }
};

template <>
struct AccChain<13, 10> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %23, %23;\n\t"
            "xor.b32 t, %13, %23;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %23;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %23;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %16, %23;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %17, %23;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %18, %23;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %19, %23;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %20, %23;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %21, %23;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "xor.b32 t, %22, %23;\n\t"
            "addc.cc.u32 %9, %9, t;\n\t"
            "addc.cc.u32 %10, %10, %23;\n\t"
            "addc.cc.u32 %11, %11, %23;\n\t"
            "addc.u32 %12, %12, %23;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(m));
    }
};

template <>
struct AccChain<13, 11> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %24, %24;\n\t"
            "xor.b32 t, %13, %24;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %24;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %24;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %16, %24;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %17, %24;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %18, %24;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %19, %24;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %20, %24;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %21, %24;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "xor.b32 t, %22, %24;\n\t"
            "addc.cc.u32 %9, %9, t;\n\t"
            "xor.b32 t, %23, %24;\n\t"
            "addc.cc.u32 %10, %10, t;\n\t"
            "addc.cc.u32 %11, %11, %24;\n\t"
            "addc.u32 %12, %12, %24;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(P[10]), "r"(m));
    }
};

template <>
struct AccChain<13, 12> {
    static __device__ __forceinline__ void add(uint32_t *acc, const uint32_t *P, uint32_t m) {
        asm("{\n\t"
            ".reg .u32 t;\n\t"
            "add.cc.u32 t, %25, %25;\n\t"
            "xor.b32 t, %13, %25;\n\t"
            "addc.cc.u32 %0, %0, t;\n\t"
            "xor.b32 t, %14, %25;\n\t"
            "addc.cc.u32 %1, %1, t;\n\t"
            "xor.b32 t, %15, %25;\n\t"
            "addc.cc.u32 %2, %2, t;\n\t"
            "xor.b32 t, %16, %25;\n\t"
            "addc.cc.u32 %3, %3, t;\n\t"
            "xor.b32 t, %17, %25;\n\t"
            "addc.cc.u32 %4, %4, t;\n\t"
            "xor.b32 t, %18, %25;\n\t"
            "addc.cc.u32 %5, %5, t;\n\t"
            "xor.b32 t, %19, %25;\n\t"
            "addc.cc.u32 %6, %6, t;\n\t"
            "xor.b32 t, %20, %25;\n\t"
            "addc.cc.u32 %7, %7, t;\n\t"
            "xor.b32 t, %21, %25;\n\t"
            "addc.cc.u32 %8, %8, t;\n\t"
            "xor.b32 t, %22, %25;\n\t"
            "addc.cc.u32 %9, %9, t;\n\t"
            "xor.b32 t, %23, %25;\n\t"
            "addc.cc.u32 %10, %10, t;\n\t"
            "xor.b32 t, %24, %25;\n\t"
            "addc.cc.u32 %11, %11, t;\n\t"
            "addc.u32 %12, %12, %25;\n\t"
            "}"
            : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
            : "r"(P[0]), "r"(P[1]), "r"(P[2]), "r"(P[3]), "r"(P[4]), "r"(P[5]), "r"(P[6]), "r"(P[7]), "r"(P[8]), "r"(P[9]), "r"(P[10]), "r"(P[11]), "r"(m));
    }
};

}  // namespace pg
