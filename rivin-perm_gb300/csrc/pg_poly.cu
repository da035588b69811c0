// Affine-polynomial Glynn: the coefficients of per(C + x L) modulo many odd
// moduli in one launch.
//
//   per(C + x L) = 2^(1-n) sum_d (prod_k d_k) prod_i (c_i(d) + x l_i(d)),
//   c_i(d) = sum_j d_j c_ij,  l_i(d) = sum_j d_j l_ij,  d_n = +1 fixed
// (rivin-perm perm_polynomial.py:268-329; native engine
// perm_polynomial_omp.c:434-486 term, 612-636 traversal, 681-779 driver).
// The principal-permanent polynomial per(I + x A) and the rook polynomials
// per(J + x A) / (n-k)! are this with C = I or C = J.
//
// GB300 organisation: the traversal is the residue kernel's — aligned Gray
// chunks of 2^log_len states, a contiguous balanced chunk range per thread,
// the column tables of C and L in shared memory (every lane of a warp toggles
// the same column inside a chunk, so reads are broadcasts), all moduli in
// one grid (grid.y = modulus).  Per state a thread multiplies the n linear
// factors into an (n+1)-coefficient vector held in registers; each
// coefficient update a*c + b*l is two 32x32->64 products summed and ONE
// Montgomery reduction (odd modulus p < 2^30 keeps the sum below p * 2^32
// and every value below 2p, so no conditional subtraction).  Coefficients
// are added into per-thread residues, reduced per block, and each block adds
// one 64-bit word per coefficient into global memory.
#include "pg_internal.h"
#include "glynn_m32.cuh"
#include "poly_common.cuh"

// 1: matrices C with equal rows (rook polynomials) take the uniform kernel.
#ifndef PG_POLY_UNIFORM
#define PG_POLY_UNIFORM 1
#endif

#include <cstring>
#include <vector>

namespace pg {

// (a*c + b*l) * 2^-32 mod p for a, b < 2p and c, l < p < 2^30: < 2p.
__device__ __forceinline__ uint32_t poly_redc2(uint32_t a, uint32_t c, uint32_t b, uint32_t l,
                                               uint32_t p, uint32_t pinv) {
    const uint64_t t = (uint64_t)a * c + (uint64_t)b * l;
    const uint32_t m = (uint32_t)t * pinv;
    return (uint32_t)(((uint64_t)m * p + t) >> 32);
}

template <int N>
__global__ void __launch_bounds__(poly_block(N)) affine_m32_kernel(PolyArgs a) {
    constexpr int NP = (N + 3) & ~3;
    constexpr int NCOL = N - 1;
    constexpr bool ACC_SM = poly_acc_in_smem(N);
    constexpr int BT = poly_block(N);
    extern __shared__ uint4 psm[];
    uint32_t *tab = reinterpret_cast<uint32_t *>(psm);
    uint32_t *accs = tab + NCOL * 4 * NP;   // [N+1][BT] when ACC_SM
    const int k = blockIdx.y;
    {
        const uint4 *g = reinterpret_cast<const uint4 *>(a.tabs + (size_t)k * NCOL * 4 * NP);
        for (int i = threadIdx.x; i < NCOL * 4 * NP / 4; i += blockDim.x) psm[i] = g[i];
    }
    const uint32_t p = a.moduli[k], pinv = a.pinvs[k];

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

    uint32_t cs[N], ls[N];
    if (c_begin < c_end) {
        const uint32_t *init = a.init + (size_t)k * 2 * NP;
#pragma unroll
        for (int i = 0; i < N; i++) {
            cs[i] = init[i];
            ls[i] = init[NP + i];
        }
        const uint64_t start = c_begin << a.log_len;
        const uint64_t gstart = start ^ (start >> 1);
        for (int j = 0; j < NCOL; j++) {
            if ((gstart >> j) & 1) {
                const uint32_t *col = tab + (4 * j + 2) * NP;   // subtract direction
#pragma unroll
                for (int i = 0; i < N; i++) {
                    cs[i] = m32_addmod(cs[i], col[i], p);
                    ls[i] = m32_addmod(ls[i], col[NP + i], p);
                }
            }
        }
    }

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
                const uint4 *col = reinterpret_cast<const uint4 *>(tab + (4 * j + 2 * sub) * NP);
#pragma unroll
                for (int v = 0; v < NP / 4; v++) {
                    const uint4 dc = col[v], dl = col[NP / 4 + v];
                    if (4 * v + 0 < N) { cs[4 * v + 0] = m32_addmod(cs[4 * v + 0], dc.x, p); ls[4 * v + 0] = m32_addmod(ls[4 * v + 0], dl.x, p); }
                    if (4 * v + 1 < N) { cs[4 * v + 1] = m32_addmod(cs[4 * v + 1], dc.y, p); ls[4 * v + 1] = m32_addmod(ls[4 * v + 1], dl.y, p); }
                    if (4 * v + 2 < N) { cs[4 * v + 2] = m32_addmod(cs[4 * v + 2], dc.z, p); ls[4 * v + 2] = m32_addmod(ls[4 * v + 2], dl.z, p); }
                    if (4 * v + 3 < N) { cs[4 * v + 3] = m32_addmod(cs[4 * v + 3], dc.w, p); ls[4 * v + 3] = m32_addmod(ls[4 * v + 3], dl.w, p); }
                }
            }
            // prod_i (c_i + x l_i): factor 0 as is, factors 1..N-1 each with
            // one Montgomery reduction per coefficient (R^-(N-1) overall)
            uint32_t P[N + 1];
            P[0] = cs[0];
            P[1] = ls[0];
#pragma unroll
            for (int r = 1; r < N; r++) {
                P[r + 1] = poly_redc2(P[r], ls[r], 0u, 0u, p, pinv);
#pragma unroll
                for (int d = r; d >= 1; d--) P[d] = poly_redc2(P[d], cs[r], P[d - 1], ls[r], p, pinv);
                P[0] = poly_redc2(P[0], cs[r], 0u, 0u, p, pinv);
            }
            // Glynn sign (-1)^popcount(gray(g)) = (-1)^(g & 1)
            const bool neg = g & 1;
#pragma unroll
            for (int d = 0; d <= N; d++) {
                const uint32_t v = __viaddmin_u32(P[d], 0u - p, P[d]);   // < p
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
    __shared__ unsigned long long red[BT / 32][N + 1];
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
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][d] = v;
    }
    __syncthreads();
    for (int d = threadIdx.x; d <= N; d += blockDim.x) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w][d];
        atomicAdd(a.acc + (size_t)k * (N + 1) + d, t);
    }
    if (threadIdx.x == 0 && any_abort) atomicExch(a.status, 1);
}

template <int N>
static cudaError_t launch_affine_n(const PolyArgs &args, int k, int sm_count, cudaStream_t s) {
    constexpr int NP = (N + 3) & ~3;
    constexpr int BT = poly_block(N);
    const size_t smem = (size_t)(N - 1) * 4 * NP * 4 +
                        (poly_acc_in_smem(N) ? (size_t)(N + 1) * BT * 4 : 0);
    cudaError_t e = cudaFuncSetAttribute(affine_m32_kernel<N>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, affine_m32_kernel<N>, BT, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    // one resident wave shared by the k moduli, no more blocks than chunks
    uint64_t bpm = ((uint64_t)per_sm * sm_count + k - 1) / k;
    const uint64_t max_blocks = (args.chunks + BT - 1) / BT;
    if (bpm > max_blocks) bpm = max_blocks;
    if (bpm < 1) bpm = 1;
    dim3 grid((unsigned)bpm, (unsigned)k);
    affine_m32_kernel<N><<<grid, BT, smem, s>>>(args);
    return cudaGetLastError();
}

static cudaError_t launch_affine(int n, const PolyArgs &args, int k, int sm_count,
                                 cudaStream_t s) {
    switch (n) {
#define PG_POLY_CASE(NN) case NN: return launch_affine_n<NN>(args, k, sm_count, s);
        PG_POLY_CASE(2) PG_POLY_CASE(3) PG_POLY_CASE(4) PG_POLY_CASE(5) PG_POLY_CASE(6)
        PG_POLY_CASE(7) PG_POLY_CASE(8) PG_POLY_CASE(9) PG_POLY_CASE(10) PG_POLY_CASE(11)
        PG_POLY_CASE(12) PG_POLY_CASE(13) PG_POLY_CASE(14) PG_POLY_CASE(15) PG_POLY_CASE(16)
        PG_POLY_CASE(17) PG_POLY_CASE(18) PG_POLY_CASE(19) PG_POLY_CASE(20) PG_POLY_CASE(21)
        PG_POLY_CASE(22) PG_POLY_CASE(23) PG_POLY_CASE(24) PG_POLY_CASE(25) PG_POLY_CASE(26)
        PG_POLY_CASE(27) PG_POLY_CASE(28) PG_POLY_CASE(29) PG_POLY_CASE(30) PG_POLY_CASE(31)
        PG_POLY_CASE(32)
#undef PG_POLY_CASE
    default:
        return cudaErrorInvalidValue;
    }
}

static size_t poly_align(size_t v) { return (v + 255) / 256 * 256; }

// True when every row of C equals the first (the rook case C = J): the
// uniform kernel of pg_poly_uniform.cu then applies.
static bool rows_equal(const int64_t *C, int n) {
    for (int i = 1; i < n; i++)
        for (int j = 0; j < n; j++)
            if (C[(size_t)i * n + j] != C[j]) return false;
    return true;
}

// The uniform kernel's launch: tables of L (Montgomery residues) plus the
// common row sum of C, one R removed at the end.
static int uniform_residues_impl(const int64_t *C, const int64_t *L, int n,
                                 const uint64_t *moduli, int k, uint64_t *out) {
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    const int NPU = poly_uniform_stride(n), NCOL = n - 1;
    const size_t tab_words = (size_t)NCOL * 2 * NPU;
    const size_t off_init = poly_align((size_t)k * tab_words * 4);
    const size_t off_mod = poly_align(off_init + (size_t)k * NPU * 4);
    const size_t off_pinv = poly_align(off_mod + (size_t)k * 4);
    const size_t off_acc = poly_align(off_pinv + (size_t)k * 4);
    const size_t off_status = poly_align(off_acc + (size_t)k * (n + 1) * 8);
    const size_t total = poly_align(off_status + 16);
    Workspace *ws;
    st = workspace(&ws, total, total);
    if (st != PG_OK) return st;
    char *h = (char *)ws->host;
    char *d = (char *)ws->dev;
    std::memset(h, 0, total);
    for (int t = 0; t < k; t++) {
        const uint64_t p = moduli[t];
        const uint64_t R = (1ull << 32) % p;
        const auto mont = [&](uint64_t x) { return (uint32_t)mulmod_u64(x % p, R, p); };
        uint32_t *tt = (uint32_t *)h + (size_t)t * tab_words;
        uint32_t *init = (uint32_t *)(h + off_init) + (size_t)t * NPU;
        // entry n of a row: the common row sum of C (row 0)
        for (int i = 0; i <= n; i++) {
            const int64_t *row = i < n ? L + (size_t)i * n : C;
            uint64_t sum = 0;
            for (int j = 0; j < n; j++) {
                const uint64_t v = normmod_i64(row[j], p);
                sum = (sum + v) % p;
                if (j < NCOL) {
                    const uint32_t v2 = mont(2 * v % p);
                    // direction 0 (column back to +): add 2a; 1 (to -): subtract 2a
                    tt[(2 * j + 0) * NPU + i] = v2 - (uint32_t)p;
                    tt[(2 * j + 1) * NPU + i] = 0u - v2;
                }
            }
            init[i] = mont(sum);
        }
        ((uint32_t *)(h + off_mod))[t] = (uint32_t)p;
        ((uint32_t *)(h + off_pinv))[t] = neg_inv32((uint32_t)p);
    }
    const ChunkPlan pl = plan_chunks(n - 1, n - 1 < 6 ? n - 1 : 6, 1ull << 20);
    PolyArgs a;
    a.tabs = (const uint32_t *)d;
    a.init = (const uint32_t *)(d + off_init);
    a.moduli = (const uint32_t *)(d + off_mod);
    a.pinvs = (const uint32_t *)(d + off_pinv);
    a.acc = (unsigned long long *)(d + off_acc);
    a.status = (int *)(d + off_status);
    a.abort_flag = abort_dev;
    a.chunks = pl.chunks;
    a.log_len = pl.log_len;
    PG_CUDA(cudaMemcpyAsync(d, h, off_acc, cudaMemcpyHostToDevice, ws->stream));
    PG_CUDA(cudaMemsetAsync(d + off_acc, 0, total - off_acc, ws->stream));
    PG_CUDA(launch_poly_uniform(n, a, k, dev.sm_count, ws->stream));
    PG_CUDA(cudaMemcpyAsync(h + off_acc, d + off_acc, total - off_acc, cudaMemcpyDeviceToHost,
                            ws->stream));
    PG_CUDA(cudaStreamSynchronize(ws->stream));
    if (*(int *)(h + off_status)) return fail(PG_EABORT, "launch aborted by pg_abort()");
    const unsigned long long *acc = (const unsigned long long *)(h + off_acc);
    for (int t = 0; t < k; t++) {
        const uint64_t p = moduli[t];
        // remove R = 2^32 (the values are Montgomery residues) and scale by
        // 2^(1-n): multiply by 2^-(n+31), 2^-1 = (p+1)/2 for odd p
        const uint64_t fix = powmod_u64((p >> 1) + 1, (uint64_t)(n + 31), p);
        for (int dgr = 0; dgr <= n; dgr++)
            out[(size_t)t * (n + 1) + dgr] = mulmod_u64(acc[(size_t)t * (n + 1) + dgr] % p, fix, p);
    }
    return PG_OK;
}

// out[t*(n+1) + d] = coefficient d of per(C + x L) mod moduli[t], 2 <= n <= 63
// (orders above 32 in pg_poly_wide.cu), odd moduli 3 <= m < 2^30, k <= 65535.
static int affine_residues_impl(const int64_t *C, const int64_t *L, int n,
                                const uint64_t *moduli, int k, uint64_t *out) {
    if (n > POLY_REG_MAX_N)
        return affine_wide_residues(C, L, n, 0, 1ull << (n - 1), true, moduli, k, out);
#if PG_POLY_UNIFORM
    if (rows_equal(C, n)) return uniform_residues_impl(C, L, n, moduli, k, out);
#endif
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    const int NP = (n + 3) & ~3, NCOL = n - 1;
    const size_t tab_words = (size_t)NCOL * 4 * NP;
    const size_t off_init = poly_align((size_t)k * tab_words * 4);
    const size_t off_mod = poly_align(off_init + (size_t)k * 2 * NP * 4);
    const size_t off_pinv = poly_align(off_mod + (size_t)k * 4);
    const size_t off_acc = poly_align(off_pinv + (size_t)k * 4);
    const size_t off_status = poly_align(off_acc + (size_t)k * (n + 1) * 8);
    const size_t total = poly_align(off_status + 16);
    Workspace *ws;
    st = workspace(&ws, total, total);
    if (st != PG_OK) return st;
    char *h = (char *)ws->host;
    char *d = (char *)ws->dev;
    std::memset(h, 0, total);
    for (int t = 0; t < k; t++) {
        const uint64_t p = moduli[t];
        uint32_t *tt = (uint32_t *)h + (size_t)t * tab_words;
        uint32_t *init = (uint32_t *)(h + off_init) + (size_t)t * 2 * NP;
        for (int i = 0; i < n; i++) {
            uint64_t sc = 0, sl = 0;
            for (int j = 0; j < n; j++) {
                const uint64_t cij = normmod_i64(C[(size_t)i * n + j], p);
                const uint64_t lij = normmod_i64(L[(size_t)i * n + j], p);
                sc = (sc + cij) % p;
                sl = (sl + lij) % p;
                if (j < NCOL) {
                    const uint32_t c2 = (uint32_t)(2 * cij % p), l2 = (uint32_t)(2 * lij % p);
                    // direction 0 (column back to +): add 2a; 1 (to -): subtract 2a
                    tt[(4 * j + 0) * NP + i] = c2 - (uint32_t)p;
                    tt[(4 * j + 1) * NP + i] = l2 - (uint32_t)p;
                    tt[(4 * j + 2) * NP + i] = 0u - c2;
                    tt[(4 * j + 3) * NP + i] = 0u - l2;
                }
            }
            init[i] = (uint32_t)sc;
            init[NP + i] = (uint32_t)sl;
        }
        ((uint32_t *)(h + off_mod))[t] = (uint32_t)p;
        ((uint32_t *)(h + off_pinv))[t] = neg_inv32((uint32_t)p);
    }
    // up to 2^20 chunks of >= 64 states per modulus over one wave of threads
    const ChunkPlan pl = plan_chunks(n - 1, n - 1 < 6 ? n - 1 : 6, 1ull << 20);
    PolyArgs a;
    a.tabs = (const uint32_t *)d;
    a.init = (const uint32_t *)(d + off_init);
    a.moduli = (const uint32_t *)(d + off_mod);
    a.pinvs = (const uint32_t *)(d + off_pinv);
    a.acc = (unsigned long long *)(d + off_acc);
    a.status = (int *)(d + off_status);
    a.abort_flag = abort_dev;
    a.chunks = pl.chunks;
    a.log_len = pl.log_len;
    PG_CUDA(cudaMemcpyAsync(d, h, off_acc, cudaMemcpyHostToDevice, ws->stream));
    PG_CUDA(cudaMemsetAsync(d + off_acc, 0, total - off_acc, ws->stream));
    PG_CUDA(launch_affine(n, a, k, dev.sm_count, ws->stream));
    PG_CUDA(cudaMemcpyAsync(h + off_acc, d + off_acc, total - off_acc, cudaMemcpyDeviceToHost,
                            ws->stream));
    PG_CUDA(cudaStreamSynchronize(ws->stream));
    if (*(int *)(h + off_status)) return fail(PG_EABORT, "launch aborted by pg_abort()");
    const unsigned long long *acc = (const unsigned long long *)(h + off_acc);
    for (int t = 0; t < k; t++) {
        const uint64_t p = moduli[t];
        // remove R^-(n-1) from the Montgomery products and scale by 2^(1-n)
        const uint64_t fix = mulmod_u64(powmod_u64((1ull << 32) % p, (uint64_t)(n - 1), p),
                                        powmod_u64((p >> 1) + 1, (uint64_t)(n - 1), p), p);
        for (int dgr = 0; dgr <= n; dgr++)
            out[(size_t)t * (n + 1) + dgr] = mulmod_u64(acc[(size_t)t * (n + 1) + dgr] % p, fix, p);
    }
    return PG_OK;
}

}  // namespace pg

extern "C" int pg_affine_residues(const int64_t *C, const int64_t *L, int n,
                                  const uint64_t *moduli, int k, uint64_t *out) {
    using namespace pg;
    if (n < 0 || n > POLY_MAX_N) return fail(PG_ERANGE, "n must satisfy 0 <= n <= 63");
    if (k < 0) return fail(PG_EINVAL, "k must be non-negative");
    if (k == 0) return PG_OK;
    if (!moduli || !out || (n > 0 && (!C || !L))) return fail(PG_EINVAL, "null argument");
    for (int t = 0; t < k; t++)
        if (moduli[t] < 3 || !(moduli[t] & 1) || moduli[t] >= (1ull << 30))
            return fail(PG_ERANGE, "moduli must be odd with 3 <= m < 2^30");
    if (n == 0) {
        for (int t = 0; t < k; t++) out[t] = 1;
        return PG_OK;
    }
    if (n == 1) {
        for (int t = 0; t < k; t++) {
            out[2 * t] = normmod_i64(C[0], moduli[t]);
            out[2 * t + 1] = normmod_i64(L[0], moduli[t]);
        }
        return PG_OK;
    }
    for (int t0 = 0; t0 < k; t0 += 65535) {
        const int kk = k - t0 < 65535 ? k - t0 : 65535;
        const int st = affine_residues_impl(C, L, n, moduli + t0, kk, out + (size_t)t0 * (n + 1));
        if (st != PG_OK) return st;
    }
    return PG_OK;
}
