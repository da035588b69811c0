// FP64-accurate Glynn permanent (forward) of real or complex matrices of any
// order 2..63, over a Gray window [g_lo, g_lo + g_count) of every matrix.
//
//   sum_{g in window} (-1)^g prod_i s_i(g),   s_i(g) = sum_j d_j(g) a_ij
// (rivin-perm permanent_glynn_kernel, perm_parallel_cuda.cu:68-209, over
// the whole walk: per(A) = 2^(1-n) times the sum over [0, 2^(n-1))).
//
// GB300 design (orders above 32 and windows; orders up to 32 with the
// gradient live in pg_f64.cu):
//   * one warp walks one contiguous part of the window of one matrix; lane l
//     owns rows l and l + 32 and keeps their double-float sums (FP32 pipes);
//   * the column table of the matrix (2 a_ij, scaled rows) sits once in
//     shared memory for the block's warps (every warp of a block works on
//     the same matrix); a step reads one entry per owned row;
//   * the lane multiplies its rows, then a shuffle butterfly multiplies the
//     lanes' products: every lane ends with the full term;
//   * rows are scaled by powers of two so that sum_j |a_ij| lies in
//     [1/2, 1): every |s_i| <= 1 and every term <= 1.  Each lane also
//     multiplies its product by 2^3 (exact), 2^96 for 32 lanes: dense
//     orders near 63 have dominant terms near 2^-200, below FP32's range,
//     which the shift lifts to about 2^-104 while the largest possible term
//     (2^96) and a block's sum (2^108) stay far below FP32's maximum;
//   * every 2^log_block states the row sums are recomputed exactly in FP64
//     and the block's double-float sum is added into FP64 Kahan sums; a
//     reduction kernel combines each matrix's warp slots in a fixed order
//     and removes the row scaling, the shift and (whole walks) 2^(n-1).
#pragma once

#include <stdint.h>

#include "df_arith.cuh"

namespace pg {

struct WideArgs {
    const double *Are, *Aim;   // [batch][n][n] row-major, device; Aim null when real
    int batch, log_w;          // 2^log_w warps per matrix
    int wpb;                   // warps per block, divides 2^log_w
    int log_block;             // exact re-initialisation period 2^log_block
    uint64_t g_lo, g_count;    // Gray window of every matrix
    double *slots;             // [batch << log_w][WIDE_SLOT]
    volatile const int *abort_flag;
    int *status;
};

constexpr int WIDE_SLOT = 8;   // re sum, re comp, im sum, im comp, sum |term|

__host__ __device__ constexpr int wide_lev(int N) {
    return N <= 2 ? 1 : N <= 4 ? 2 : N <= 8 ? 3 : N <= 16 ? 4 : 5;
}
// log2 of the power-of-two factor every term carries (3 per butterfly lane)
__host__ __device__ constexpr int wide_shift(int N) { return 3 << wide_lev(N); }

__device__ __forceinline__ df df_scale8(df a) { return df{a.hi * 8.f, a.lo * 8.f}; }

template <int N, bool CPLX>
__global__ void __launch_bounds__(128) glynn_wide_kernel(WideArgs a) {
    constexpr int R = N > 32 ? 2 : 1;          // rows per lane
    constexpr int NP = 32 * R;
    constexpr int LEV = wide_lev(N);
    extern __shared__ __align__(16) unsigned char wide_smem[];
    df *tre = reinterpret_cast<df *>(wide_smem);   // [N-1][NP]
    df *tim = tre + (N - 1) * NP;                  // complex only
    __shared__ double rsc[NP];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const long first = (long)blockIdx.x * a.wpb;
    const int b = (int)(first >> a.log_w);
    const double *Ar = a.Are + (size_t)b * N * N;
    const double *Ai = CPLX ? a.Aim + (size_t)b * N * N : nullptr;

    for (int r = threadIdx.x; r < NP; r += blockDim.x) {
        double rowsum = 0.0;
        if (r < N)
            for (int j = 0; j < N; j++)
                rowsum += fabs(Ar[r * N + j]) + (CPLX ? fabs(Ai[r * N + j]) : 0.0);
        int ex = 0;
        if (rowsum > 0.0) { frexp(rowsum, &ex); ex = -ex; }
        rsc[r] = ldexp(1.0, ex);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < (N - 1) * NP; idx += blockDim.x) {
        const int j = idx / NP, r = idx % NP;
        tre[idx] = r < N ? df_from(2.0 * Ar[r * N + j] * rsc[r]) : df{0.f, 0.f};
        if (CPLX) tim[idx] = r < N ? df_from(2.0 * Ai[r * N + j] * rsc[r]) : df{0.f, 0.f};
    }
    __syncthreads();

    // this warp's balanced part of the window
    const uint64_t W = 1ull << a.log_w;
    const uint64_t part = (uint64_t)(first + wib) & (W - 1);
    const uint64_t base = a.g_count >> a.log_w, rem = a.g_count & (W - 1);
    const uint64_t g_begin = a.g_lo + part * base + (part < rem ? part : rem);
    const uint64_t g_end = g_begin + base + (part < rem ? 1 : 0);
    const uint64_t block_len = 1ull << a.log_block;

    double sre = 0.0, cre = 0.0, sim = 0.0, cim = 0.0, asum = 0.0;
    bool aborted = false;
    for (uint64_t g0 = g_begin; g0 < g_end; g0 += block_len) {
        if (*a.abort_flag) { aborted = true; break; }
        const uint64_t g1 = g_end - g0 < block_len ? g_end : g0 + block_len;
        // exact FP64 row sums at g0 (rows beyond N: s = 1, table entries 0)
        const uint64_t gr = g0 ^ (g0 >> 1);
        df s_re[R], s_im[R];
#pragma unroll
        for (int k = 0; k < R; k++) {
            const int r = lane + 32 * k;
            double vr = 0.0, vi = 0.0;
            if (r < N) {
                for (int j = 0; j < N; j++) {
                    const bool neg = j < N - 1 && ((gr >> j) & 1);
                    const double xr = Ar[r * N + j] * rsc[r];
                    vr += neg ? -xr : xr;
                    if (CPLX) {
                        const double xi = Ai[r * N + j] * rsc[r];
                        vi += neg ? -xi : xi;
                    }
                }
                s_re[k] = df_from(vr);
                s_im[k] = df_from(vi);
            } else {
                s_re[k] = df{1.f, 0.f};
                s_im[k] = df{0.f, 0.f};
            }
        }
        df bre = df{0.f, 0.f}, bim = df{0.f, 0.f};
        float babs = 0.f;
        for (uint64_t g = g0; g < g1; g++) {
            if (g != g0) {
                const int j = __ffsll((long long)g) - 1;
                const bool sub = ((g >> (j + 1)) & 1) == 0;
#pragma unroll
                for (int k = 0; k < R; k++) {
                    const df dr = tre[j * NP + lane + 32 * k];
                    s_re[k] = df_add(s_re[k], sub ? df_neg(dr) : dr);
                    if (CPLX) {
                        const df di = tim[j * NP + lane + 32 * k];
                        s_im[k] = df_add(s_im[k], sub ? df_neg(di) : di);
                    }
                }
            }
            if (CPLX) {
                dc P = dc{s_re[0], s_im[0]};
                if (R > 1) P = dc_mul(P, dc{s_re[R - 1], s_im[R - 1]});
                P = dc{df_scale8(P.re), df_scale8(P.im)};
#pragma unroll
                for (int lv = 0; lv < LEV; lv++)
                    P = dc_mul(P, dc{df_shfl_xor(P.re, 1 << lv), df_shfl_xor(P.im, 1 << lv)});
                if (g & 1) P = dc{df_neg(P.re), df_neg(P.im)};
                bre = df_add(bre, P.re);
                bim = df_add(bim, P.im);
                babs += hypotf(P.re.hi, P.im.hi);
            } else {
                df P = s_re[0];
                if (R > 1) P = df_mul(P, s_re[R - 1]);
                P = df_scale8(P);
#pragma unroll
                for (int lv = 0; lv < LEV; lv++) P = df_mul(P, df_shfl_xor(P, 1 << lv));
                if (g & 1) P = df_neg(P);
                bre = df_add(bre, P);
                babs += fabsf(P.hi);
            }
        }
        kahan(sre, cre, df_to(bre));
        if (CPLX) kahan(sim, cim, df_to(bim));
        asum += (double)babs;
    }
    if (lane == 0) {
        double *slot = a.slots + (size_t)(first + wib) * WIDE_SLOT;
        slot[0] = sre; slot[1] = cre; slot[2] = sim; slot[3] = cim; slot[4] = asum;
        if (aborted) atomicExch(a.status, 1);
    }
}

template <int N, bool CPLX>
cudaError_t launch_glynn_wide(const WideArgs &a, cudaStream_t s) {
    constexpr int NP = 32 * (N > 32 ? 2 : 1);
    const size_t smem = (size_t)(N - 1) * NP * sizeof(df) * (CPLX ? 2 : 1);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(glynn_wide_kernel<N, CPLX>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    const long warps = (long)a.batch << a.log_w;
    glynn_wide_kernel<N, CPLX><<<(unsigned)(warps / a.wpb), 32 * a.wpb, smem, s>>>(a);
    return cudaGetLastError();
}

// Instantiated in f64_wide_{r,c}{lo,hi}.cu: orders 2..32 and 33..63.
cudaError_t launch_glynn_wide_real_lo(int n, const WideArgs &a, cudaStream_t s);
cudaError_t launch_glynn_wide_real_hi(int n, const WideArgs &a, cudaStream_t s);
cudaError_t launch_glynn_wide_cplx_lo(int n, const WideArgs &a, cudaStream_t s);
cudaError_t launch_glynn_wide_cplx_hi(int n, const WideArgs &a, cudaStream_t s);

// Host driver: Gray window [lo, lo + count) of each of `batch` matrices
// (device planes; Aim null for real), results into device arrays re/im/abs
// (im, abs nullable).  whole: also divide by 2^(n-1) (count must then be
// the whole walk).  Synchronises the stream.
int glynn_wide_run(const double *Are, const double *Aim, int batch, int n, uint64_t lo,
                   uint64_t count, bool whole, double *re, double *im, double *abs_sum,
                   cudaStream_t stream);

}  // namespace pg
