// Affine-polynomial Glynn for orders 33..63 and for Gray windows of any
// order: the coefficients of per(C + x L) modulo many odd moduli, summed
// over the states [lo, hi) of the walk (the whole walk: 2^(n-1) per(C + xL)).
//
// Same algorithm, tables and Montgomery arithmetic as affine_m32_kernel
// (pg_poly.cu; rivin-perm perm_polynomial.py:268-329 and
// perm_polynomial_omp.c:612-636), with the order a runtime value: the
// per-thread row sums c_i, l_i, the coefficient vector P and the
// coefficient accumulators live in shared memory (thread-minor, so a warp
// touches 32 consecutive banks), which keeps one kernel for every order and
// the product loop triangular (factor r updates coefficients r+1..0, one
// shared load and one store per Montgomery reduction).  The column tables
// stay in global memory: inside an aligned chunk every lane of a warp reads
// the same table row, a broadcast served by L1.  Orders this large take
// minutes to hours per modulus; the tests run windows.
#include "pg_internal.h"
#include "glynn_m32.cuh"
#include "poly_common.cuh"

#include <cstring>
#include <vector>

namespace pg {

constexpr int POLY_WIDE_BT = 64;

// (a*c + b*l) * 2^-32 mod p for a, b < 2p and c, l < p < 2^30: < 2p.
__device__ __forceinline__ uint32_t pw_redc2(uint32_t a, uint32_t c, uint32_t b, uint32_t l,
                                             uint32_t p, uint32_t pinv) {
    const uint64_t t = (uint64_t)a * c + (uint64_t)b * l;
    const uint32_t m = (uint32_t)t * pinv;
    return (uint32_t)(((uint64_t)m * p + t) >> 32);
}

__global__ void __launch_bounds__(POLY_WIDE_BT) affine_wide_kernel(PolyArgs a, int n) {
    constexpr int BT = POLY_WIDE_BT;
    const int NP = (n + 3) & ~3, NCOL = n - 1;
    extern __shared__ uint32_t pwsm[];
    uint32_t *cs = pwsm;                      // [n][BT]
    uint32_t *ls = cs + n * BT;               // [n][BT]
    uint32_t *P = ls + n * BT;                // [n+1][BT]
    uint32_t *acc = P + (n + 1) * BT;         // [n+1][BT]
    const int t = threadIdx.x;
    const int k = blockIdx.y;
    const uint32_t *tab = a.tabs + (size_t)k * NCOL * 4 * NP;
    const uint32_t p = a.moduli[k], pinv = a.pinvs[k];
    for (int d = 0; d <= n; d++) acc[d * BT + t] = 0;

    const uint64_t T = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + t;
    const uint64_t c_begin = a.chunk0 + tid * a.chunks / T;
    const uint64_t c_end = a.chunk0 + (tid + 1) * a.chunks / T;
    bool aborted = false;
    if (c_begin < c_end) {
        const uint32_t *init = a.init + (size_t)k * 2 * NP;
        for (int i = 0; i < n; i++) {
            cs[i * BT + t] = init[i];
            ls[i * BT + t] = init[NP + i];
        }
        const uint64_t start = c_begin << a.log_len;
        const uint64_t gstart = start ^ (start >> 1);
        for (int j = 0; j < NCOL; j++) {
            if ((gstart >> j) & 1) {
                const uint32_t *col = tab + (4 * j + 2) * NP;   // subtract direction
                for (int i = 0; i < n; i++) {
                    cs[i * BT + t] = m32_addmod(cs[i * BT + t], __ldg(col + i), p);
                    ls[i * BT + t] = m32_addmod(ls[i * BT + t], __ldg(col + NP + i), p);
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
                const uint32_t *col = tab + (4 * j + 2 * sub) * NP;
#pragma unroll 4
                for (int r = 0; r < n; r++) {
                    cs[r * BT + t] = m32_addmod(cs[r * BT + t], __ldg(col + r), p);
                    ls[r * BT + t] = m32_addmod(ls[r * BT + t], __ldg(col + NP + r), p);
                }
            }
            // prod_i (c_i + x l_i): factor 0 as is, factors 1..n-1 each with
            // one Montgomery reduction per coefficient (R^-(n-1) overall)
            P[0 * BT + t] = cs[t];
            P[1 * BT + t] = ls[t];
            for (int r = 1; r < n; r++) {
                const uint32_t cr = cs[r * BT + t], lr = ls[r * BT + t];
                uint32_t hi = P[r * BT + t];
                P[(r + 1) * BT + t] = pw_redc2(hi, lr, 0u, 0u, p, pinv);
#pragma unroll 4
                for (int d = r; d >= 1; d--) {
                    const uint32_t lo = P[(d - 1) * BT + t];
                    P[d * BT + t] = pw_redc2(hi, cr, lo, lr, p, pinv);
                    hi = lo;
                }
                P[t] = pw_redc2(hi, cr, 0u, 0u, p, pinv);
            }
            // Glynn sign (-1)^popcount(gray(g)) = (-1)^(g & 1)
            const bool neg = g & 1;
            for (int d = 0; d <= n; d++) {
                const uint32_t pv = P[d * BT + t];
                const uint32_t v = __viaddmin_u32(pv, 0u - p, pv);   // < p
                acc[d * BT + t] = m32_addmod(acc[d * BT + t], neg ? 0u - v : v - p, p);
            }
        }
    }
    __syncthreads();
    // block sums per coefficient (residues < 2^30: 64-bit sums cannot overflow)
    for (int d = t; d <= n; d += BT) {
        unsigned long long s = 0;
        for (int u = 0; u < BT; u++) s += acc[d * BT + u];
        atomicAdd(a.acc + (size_t)k * (n + 1) + d, s);
    }
    if (aborted) atomicExch(a.status, 1);
}

// out[t*(n+1) + d] = coefficient d of the Glynn sum of per(C + x L) over the
// chunk-aligned states [lo, hi) mod moduli[t] (whole: scaled by 2^(1-n),
// i.e. the coefficients of per(C + x L) when [lo, hi) is the whole walk).
int affine_wide_residues(const int64_t *C, const int64_t *L, int n, uint64_t lo, uint64_t hi,
                         bool whole, const uint64_t *moduli, int k, uint64_t *out) {
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    const int log_states = n - 1;
    const uint64_t count = hi - lo;
    // chunks: aligned to the window, >= 2^min(6, ...) states, about 2^20 of
    // them per modulus
    int ll = log_states;
    while (ll > 0 && (((lo | count) & ((1ull << ll) - 1)) != 0)) ll--;
    const ChunkPlan pl = plan_chunks(log_states, log_states < 6 ? log_states : 6, 1ull << 20);
    if (pl.log_len < ll) ll = pl.log_len;
    const int NP = (n + 3) & ~3, NCOL = n - 1;
    const size_t tab_words = (size_t)NCOL * 4 * NP;
    const auto al = [](size_t v) { return (v + 255) / 256 * 256; };
    const size_t off_init = al((size_t)k * tab_words * 4);
    const size_t off_mod = al(off_init + (size_t)k * 2 * NP * 4);
    const size_t off_pinv = al(off_mod + (size_t)k * 4);
    const size_t off_acc = al(off_pinv + (size_t)k * 4);
    const size_t off_status = al(off_acc + (size_t)k * (n + 1) * 8);
    const size_t total = al(off_status + 16);
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
    PolyArgs a;
    a.tabs = (const uint32_t *)d;
    a.init = (const uint32_t *)(d + off_init);
    a.moduli = (const uint32_t *)(d + off_mod);
    a.pinvs = (const uint32_t *)(d + off_pinv);
    a.acc = (unsigned long long *)(d + off_acc);
    a.status = (int *)(d + off_status);
    a.abort_flag = abort_dev;
    a.log_len = ll;
    a.chunk0 = lo >> ll;
    a.chunks = count >> ll;
    const size_t smem = (size_t)(4 * n + 2) * POLY_WIDE_BT * 4;
    PG_CUDA(cudaFuncSetAttribute(affine_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    int per_sm = 0;
    PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, affine_wide_kernel,
                                                          POLY_WIDE_BT, smem));
    if (per_sm < 1) per_sm = 1;
    uint64_t bpm = ((uint64_t)per_sm * dev.sm_count + k - 1) / k;
    const uint64_t max_blocks = (a.chunks + POLY_WIDE_BT - 1) / POLY_WIDE_BT;
    if (bpm > max_blocks) bpm = max_blocks;
    if (bpm < 1) bpm = 1;
    PG_CUDA(cudaMemcpyAsync(d, h, off_acc, cudaMemcpyHostToDevice, ws->stream));
    PG_CUDA(cudaMemsetAsync(d + off_acc, 0, total - off_acc, ws->stream));
    affine_wide_kernel<<<dim3((unsigned)bpm, (unsigned)k), POLY_WIDE_BT, smem, ws->stream>>>(a, n);
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaMemcpyAsync(h + off_acc, d + off_acc, total - off_acc, cudaMemcpyDeviceToHost,
                            ws->stream));
    PG_CUDA(cudaStreamSynchronize(ws->stream));
    if (*(int *)(h + off_status)) return fail(PG_EABORT, "launch aborted by pg_abort()");
    const unsigned long long *acc = (const unsigned long long *)(h + off_acc);
    for (int t = 0; t < k; t++) {
        const uint64_t p = moduli[t];
        // remove R^-(n-1) from the Montgomery products; whole walks are also
        // scaled by 2^(1-n)
        uint64_t fix = powmod_u64((1ull << 32) % p, (uint64_t)(n - 1), p);
        if (whole) fix = mulmod_u64(fix, powmod_u64((p >> 1) + 1, (uint64_t)(n - 1), p), p);
        for (int dgr = 0; dgr <= n; dgr++)
            out[(size_t)t * (n + 1) + dgr] = mulmod_u64(acc[(size_t)t * (n + 1) + dgr] % p, fix, p);
    }
    return PG_OK;
}

}  // namespace pg

extern "C" int pg_affine_residues_partial(const int64_t *C, const int64_t *L, int n,
                                          uint64_t state_lo, uint64_t state_hi,
                                          const uint64_t *moduli, int k, uint64_t *out) {
    using namespace pg;
    if (n < 2 || n > POLY_MAX_N) return fail(PG_ERANGE, "n must satisfy 2 <= n <= 63");
    if (k < 0) return fail(PG_EINVAL, "k must be non-negative");
    if (k == 0) return PG_OK;
    if (!moduli || !out || !C || !L) return fail(PG_EINVAL, "null argument");
    for (int t = 0; t < k; t++)
        if (moduli[t] < 3 || !(moduli[t] & 1) || moduli[t] >= (1ull << 30))
            return fail(PG_ERANGE, "moduli must be odd with 3 <= m < 2^30");
    const uint64_t states = 1ull << (n - 1);
    if (state_lo >= state_hi || state_hi > states)
        return fail(PG_ERANGE, "state range must satisfy lo < hi <= 2^(n-1)");
    for (int t0 = 0; t0 < k; t0 += 65535) {
        const int kk = k - t0 < 65535 ? k - t0 : 65535;
        const int st = affine_wide_residues(C, L, n, state_lo, state_hi, false, moduli + t0, kk,
                                            out + (size_t)t0 * (n + 1));
        if (st != PG_OK) return st;
    }
    return PG_OK;
}
