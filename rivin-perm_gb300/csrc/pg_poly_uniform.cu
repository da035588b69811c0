// Polynomial Glynn for C with equal rows (the rook polynomials: C = J).
//
// With every row of C equal, every row's constant part is the same
// c(d) = sum_j d_j c_j, so
//   prod_i (c + x l_i(d)) = sum_k e_k(l_1(d), ..., l_n(d)) c^(n-k) x^k
// with e_k the elementary symmetric sums (the reference's rook_polynomial,
// perm_polynomial.py:1288-1411, is per(J + x A): C = J).  A state
// costs the e_k recurrence, E[d] += l_r E[d-1] with ONE Montgomery product
// per coefficient (the general kernel needs a two-product reduction), and
// 2n - 1 products for the powers of c and the weighting.  Only one copy of
// c is kept instead of n row sums of C.
//
// Values are Montgomery residues (x R mod p, R = 2^32), so a reduction of a
// product stays in that form: the table deltas and initial sums are stored
// as Montgomery residues, E[0] = R mod p, and the host removes one R at
// the end.  E[d] is kept below 2p (one conditional subtraction of 2p per
// update), inputs of a reduction are below 2p and p, so odd p < 2^30 keeps
// every sum below 2^32.  Traversal, chunking, accumulation and the block
// reduction are the general kernel's (pg_poly.cu).
#include "pg_internal.h"
#include "glynn_m32.cuh"
#include "poly_common.cuh"

namespace pg {

template <int N>
__global__ void __launch_bounds__(poly_block(N)) uniform_m32_kernel(PolyArgs a) {
    constexpr int NPU = poly_uniform_stride(N);
    constexpr int NCOL = N - 1;
    constexpr bool ACC_SM = poly_acc_in_smem(N);
    constexpr int BT = poly_block(N);
    extern __shared__ uint4 usm[];
    uint32_t *tab = reinterpret_cast<uint32_t *>(usm);
    uint32_t *accs = tab + NCOL * 2 * NPU;   // [N+1][BT] when ACC_SM
    const int k = blockIdx.y;
    {
        const uint4 *g = reinterpret_cast<const uint4 *>(a.tabs + (size_t)k * NCOL * 2 * NPU);
        for (int i = threadIdx.x; i < NCOL * 2 * NPU / 4; i += blockDim.x) usm[i] = g[i];
    }
    const uint32_t p = a.moduli[k], pinv = a.pinvs[k];
    const uint32_t one = (uint32_t)((1ull << 32) % p);   // R mod p: Montgomery 1

    uint32_t acc[ACC_SM ? 1 : N + 1];
    if constexpr (ACC_SM) {
        for (int d = 0; d <= N; d++) accs[d * BT + threadIdx.x] = 0;
    } else {
#pragma unroll
        for (int d = 0; d <= N; d++) acc[d] = 0;
    }
    __syncthreads();
    bool aborted = false;

    const uint64_t T = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t c_begin = tid * a.chunks / T;
    const uint64_t c_end = (tid + 1) * a.chunks / T;

    uint32_t ls[N], cm = 0;
    if (c_begin < c_end) {
        const uint32_t *init = a.init + (size_t)k * NPU;
#pragma unroll
        for (int i = 0; i < N; i++) ls[i] = init[i];
        cm = init[N];
        const uint64_t start = c_begin << a.log_len;
        const uint64_t gstart = start ^ (start >> 1);
        for (int j = 0; j < NCOL; j++) {
            if ((gstart >> j) & 1) {
                const uint32_t *col = tab + (2 * j + 1) * NPU;   // subtract direction
#pragma unroll
                for (int i = 0; i < N; i++) ls[i] = m32_addmod(ls[i], col[i], p);
                cm = m32_addmod(cm, col[N], p);
            }
        }
    }
    const uint32_t p2 = 2 * p;
    const auto red2p = [&](uint32_t x) { return __viaddmin_u32(x, 0u - p2, x); };   // < 4p -> < 2p
    const auto red = [&](uint32_t x) { return __viaddmin_u32(x, 0u - p, x); };      // < 2p -> < p

    const uint32_t len = 1u << a.log_len;
    // the host-mapped abort word is read once per 2^12 states (per chunk for
    // longer chunks), from the thread's second period on
    const uint64_t poll = a.log_len >= 12 ? 0 : (1ull << (12 - a.log_len)) - 1;
    for (uint64_t c = c_begin; c < c_end; c++) {
        if (c != c_begin && ((c - c_begin) & poll) == 0 && *a.abort_flag) {
            aborted = true;
            break;
        }
        for (uint32_t i = 0; i < len; i++) {
            const uint64_t g = (c << a.log_len) | i;
            if (i != 0 || c != c_begin) {
                // Gray step into state g: column j = ctz(g) flips; it turns
                // negative when bit j+1 of g is 0
                const int j = i ? __ffs(i) - 1 : a.log_len + __ffsll((long long)c) - 1;
                const int sub = ((g >> (j + 1)) & 1) == 0;
                const uint32_t *row = tab + (2 * j + sub) * NPU;
                const uint4 *col = reinterpret_cast<const uint4 *>(row);
#pragma unroll
                for (int v = 0; v < NPU / 4; v++) {
                    const uint4 dl = col[v];
                    if (4 * v + 0 < N) ls[4 * v + 0] = m32_addmod(ls[4 * v + 0], dl.x, p);
                    if (4 * v + 1 < N) ls[4 * v + 1] = m32_addmod(ls[4 * v + 1], dl.y, p);
                    if (4 * v + 2 < N) ls[4 * v + 2] = m32_addmod(ls[4 * v + 2], dl.z, p);
                    if (4 * v + 3 < N) ls[4 * v + 3] = m32_addmod(ls[4 * v + 3], dl.w, p);
                }
                cm = m32_addmod(cm, row[N], p);
            }
            // elementary symmetric sums of l_0..l_{N-1} (Montgomery, < 2p)
            uint32_t E[N + 1];
            E[0] = one;
            E[1] = ls[0];
#pragma unroll
            for (int r = 1; r < N; r++) {
                E[r + 1] = m32_redc_mul(E[r], ls[r], p, pinv);
#pragma unroll
                for (int d = r; d >= 1; d--)
                    E[d] = red2p(E[d] + m32_redc_mul(E[d - 1], ls[r], p, pinv));
            }
            // coefficient d = e_d c^(N-d): powers of c from the top down
            const bool neg = g & 1;   // Glynn sign (-1)^(g & 1)
            uint32_t pw = cm;         // c^1 (Montgomery, < p)
#pragma unroll
            for (int d = N; d >= 0; d--) {
                uint32_t v;
                if (d == N) {
                    v = red(red2p(E[N]));
                } else {
                    v = red(m32_redc_mul(E[d], pw, p, pinv));
                    if (d > 0) pw = red(m32_redc_mul(pw, cm, p, pinv));
                }
                if constexpr (ACC_SM) {
                    uint32_t &x = accs[d * BT + threadIdx.x];
                    x = m32_addmod(x, neg ? 0u - v : v - p, p);
                } else {
                    acc[d] = m32_addmod(acc[d], neg ? 0u - v : v - p, p);
                }
            }
        }
    }

    // block reduction per coefficient; residues < 2^30, so 64-bit sums over
    // the whole grid cannot overflow
    __shared__ unsigned long long red_s[BT / 32][N + 1];
    __shared__ int any_abort;
    if (threadIdx.x == 0) any_abort = 0;
    __syncthreads();
    if (aborted) any_abort = 1;
#pragma unroll
    for (int d = 0; d <= N; d++) {
        unsigned long long v;
        if constexpr (ACC_SM) v = accs[d * BT + threadIdx.x];
        else v = acc[d];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0) red_s[threadIdx.x >> 5][d] = v;
    }
    __syncthreads();
    for (int d = threadIdx.x; d <= N; d += blockDim.x) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red_s[w][d];
        atomicAdd(a.acc + (size_t)k * (N + 1) + d, t);
    }
    if (threadIdx.x == 0 && any_abort) atomicExch(a.status, 1);
}

template <int N>
static cudaError_t launch_uniform_n(const PolyArgs &args, int k, int sm_count, cudaStream_t s) {
    constexpr int NPU = poly_uniform_stride(N);
    constexpr int BT = poly_block(N);
    const size_t smem = (size_t)(N - 1) * 2 * NPU * 4 +
                        (poly_acc_in_smem(N) ? (size_t)(N + 1) * BT * 4 : 0);
    cudaError_t e = cudaFuncSetAttribute(uniform_m32_kernel<N>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, uniform_m32_kernel<N>, BT, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    uint64_t bpm = ((uint64_t)per_sm * sm_count + k - 1) / k;
    const uint64_t max_blocks = (args.chunks + BT - 1) / BT;
    if (bpm > max_blocks) bpm = max_blocks;
    if (bpm < 1) bpm = 1;
    dim3 grid((unsigned)bpm, (unsigned)k);
    uniform_m32_kernel<N><<<grid, BT, smem, s>>>(args);
    return cudaGetLastError();
}

cudaError_t launch_poly_uniform(int n, const PolyArgs &args, int k, int sm_count,
                                cudaStream_t s) {
    switch (n) {
#define PG_UNI_CASE(NN) case NN: return launch_uniform_n<NN>(args, k, sm_count, s);
        PG_UNI_CASE(2) PG_UNI_CASE(3) PG_UNI_CASE(4) PG_UNI_CASE(5) PG_UNI_CASE(6)
        PG_UNI_CASE(7) PG_UNI_CASE(8) PG_UNI_CASE(9) PG_UNI_CASE(10) PG_UNI_CASE(11)
        PG_UNI_CASE(12) PG_UNI_CASE(13) PG_UNI_CASE(14) PG_UNI_CASE(15) PG_UNI_CASE(16)
        PG_UNI_CASE(17) PG_UNI_CASE(18) PG_UNI_CASE(19) PG_UNI_CASE(20) PG_UNI_CASE(21)
        PG_UNI_CASE(22) PG_UNI_CASE(23) PG_UNI_CASE(24) PG_UNI_CASE(25) PG_UNI_CASE(26)
        PG_UNI_CASE(27) PG_UNI_CASE(28) PG_UNI_CASE(29) PG_UNI_CASE(30) PG_UNI_CASE(31)
        PG_UNI_CASE(32)
#undef PG_UNI_CASE
    default:
        return cudaErrorInvalidValue;
    }
}

}  // namespace pg
