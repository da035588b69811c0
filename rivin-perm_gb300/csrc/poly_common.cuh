// Launch arguments and shapes shared by the polynomial Glynn kernels
// (pg_poly.cu: general C + xL; pg_poly_uniform.cu: C with equal rows).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pg {

constexpr int POLY_MAX_N = 63;
// Largest order of the register kernels (pg_poly.cu, pg_poly_uniform.cu);
// larger orders and Gray windows run the shared-memory kernel of
// pg_poly_wide.cu.
constexpr int POLY_REG_MAX_N = 32;

struct PolyArgs {
    // general kernel: [k][N-1][2 dir][2 (C, L)][NP], (d - p) mod 2^32;
    // uniform kernel: [k][N-1][2 dir][NPU], L rows then the C row sum,
    // Montgomery residues, (d - p) mod 2^32
    const uint32_t *tabs;
    // general: [k][2][NP] row sums of C and L; uniform: [k][NPU]
    const uint32_t *init;
    const uint32_t *moduli;   // [k]
    const uint32_t *pinvs;    // [k]  -p^-1 mod 2^32
    unsigned long long *acc;  // [k][N+1] (zeroed)
    int *status;
    volatile const int *abort_flag;
    uint64_t chunks;          // chunks per modulus
    int log_len;
    uint64_t chunk0 = 0;      // first chunk (pg_poly_wide.cu windows)
};

// Glynn sums of per(C + x L) over the chunk-aligned Gray states [lo, hi)
// modulo odd moduli < 2^30, orders 2..63 (pg_poly_wide.cu); `whole` also
// scales by 2^(1-n).
int affine_wide_residues(const int64_t *C, const int64_t *L, int n, uint64_t lo, uint64_t hi,
                         bool whole, const uint64_t *moduli, int k, uint64_t *out);

// From order 20 on the n+1 coefficient accumulators move from registers to
// shared memory (one word per coefficient and thread, thread-minor so a warp
// touches 32 consecutive banks) and blocks shrink to 128 threads: the row
// sums and the coefficient vector alone fill most of the register file, and
// fewer registers per thread let three or more blocks share an SM.
__host__ __device__ constexpr bool poly_acc_in_smem(int N) { return N >= 20; }
__host__ __device__ constexpr int poly_block(int N) { return poly_acc_in_smem(N) ? 128 : 256; }

// Row stride of the uniform kernel's tables: N L-rows plus the C row sum,
// rounded up to 16 bytes.
__host__ __device__ constexpr int poly_uniform_stride(int N) { return (N + 4) & ~3; }

// Launches the uniform kernel for order n (pg_poly_uniform.cu).
cudaError_t launch_poly_uniform(int n, const PolyArgs &args, int k, int sm_count,
                                cudaStream_t s);

}  // namespace pg
