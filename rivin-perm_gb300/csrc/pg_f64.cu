// FP64-accurate Glynn permanent and gradient for batches of real matrices.
//
//   per(A)         = 2^(1-n) sum_d (prod_k d_k) prod_i s_i(d)
//   d per / d a_ij = 2^(1-n) sum_d (prod_k d_k) d_j prod_{l != i} s_l(d)
//                  = per(A without row i and column j)
// (forward: rivin-perm perm_parallel_cuda.cu:68-209; the gradient has no
// reference counterpart).  Row sums s_i(d) = sum_j d_j a_ij, last sign fixed.
//
// GB300 design.  FP64 issue rate on this part is a small fraction of FP32,
// so the inner loop runs in double-float arithmetic (an unevaluated sum of
// two FP32 numbers, ~48-bit significand) on the FP32 pipes:
//   * one warp walks one Gray range of one matrix; lane i owns row i
//     (n <= 32), keeps s_i, and updates it with one double-float add per
//     step from a per-warp shared-memory column table;
//   * a 5-level shuffle butterfly gives every lane both the full product
//     T = prod_l s_l and its all-but-self product E_i = prod_{l != i} s_l;
//   * gradient columns use aligned chunks of 2^M states: columns j >= M keep
//     one sign inside a chunk, so lane i adds w_i = (-1)^g E_i into W_i and,
//     for j < M, into V_ij with compile-time signs; at a chunk's end
//     G_ij += sign_j(chunk) W_i.  Per state and lane: 1 + M double-float adds.
// Accuracy: rows are pre-scaled by powers of two (exact) so row bounds are
// ~1; every 2^LOG_BLOCK states the row sums are recomputed exactly in FP64
// (bounding drift) and the block's double-float sums are added into FP64
// Kahan accumulators held in the warp's global scratch slot; a second
// kernel reduces the slots of each matrix (deterministic order).  The sum of
// |terms| is accumulated alongside, so every result carries its error scale.
#include "pg_internal.h"
#include "df_arith.cuh"
#include "f64_wide.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace pg {

// Per-warp scratch slot layout (doubles).
__host__ __device__ constexpr int f64_slot_doubles(int n) { return 4 + 2 * n * n + n; }

struct F64Args {
    const double *A;          // [batch][n][n] row-major, device
    int batch, n, log_w;      // warps per matrix = 2^log_w
    int log_block;            // exact re-initialisation period 2^log_block
    int want_grad;
    double *slots;            // [batch << log_w][slot]
    volatile const int *abort_flag;
    int *status;
};

static constexpr int F64_M = 4;                 // low gradient columns per chunk

template <int N, bool GRAD>
__global__ void __launch_bounds__(128) glynn_f64_kernel(F64Args a) {
    constexpr int LEV = N <= 2 ? 1 : N <= 4 ? 2 : N <= 8 ? 3 : N <= 16 ? 4 : 5;
    constexpr int M = (N - 1) < F64_M ? (N - 1) : F64_M;
    __shared__ df tab[4][N > 1 ? N - 1 : 1][32];   // 2 a'_ij per warp, column-major
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const long gw = (long)blockIdx.x * 4 + wib;
    if (gw >= ((long)a.batch << a.log_w)) return;
    const int b = (int)(gw >> a.log_w);
    const uint64_t part = (uint64_t)(gw & ((1 << a.log_w) - 1));
    const uint64_t states = 1ull << (N - 1);
    const uint64_t per_warp = states >> a.log_w;
    const uint64_t g_begin = part * per_warp, g_end = g_begin + per_warp;
    const double *Ab = a.A + (size_t)b * N * N;
    const bool live = lane < N;

    // power-of-two row scaling: row bound of the scaled row in [0.5, 1)
    double rowsum = 0.0;
    if (live)
        for (int j = 0; j < N; j++) rowsum += fabs(Ab[lane * N + j]);
    int ex = 0;
    if (live && rowsum > 0.0) { frexp(rowsum, &ex); ex = -ex; }
    const double rscale = ldexp(1.0, ex);
    for (int j = 0; j < N - 1; j++)
        tab[wib][j][lane] = live ? df_from(2.0 * Ab[lane * N + j] * rscale) : df{0.f, 0.f};
    __syncwarp();

    double *slot = a.slots + (size_t)gw * f64_slot_doubles(N);
    double fsum = 0.0, fcomp = 0.0, fabs_sum = 0.0;
    double gabs = 0.0;
    // Gradient columns by sign period: j < M change sign inside a chunk (V,
    // compile-time signs), M <= j < lb (lb = log_block) keep one sign per
    // chunk (GM[j - M] += +-W at each chunk's end), and j >= lb keep one sign
    // per exact-initialisation block (one block sum WB, signed at the flush;
    // the last column's sign is fixed).  Keeping per-column accumulators only
    // for j < lb frees registers and most chunk-end adds.
    constexpr int LBMAX = 12;                       // the host's largest log_block
    constexpr int NMID = (N - 1 < LBMAX ? N - 1 : LBMAX) - M > 0
                             ? (N - 1 < LBMAX ? N - 1 : LBMAX) - M : 1;
    df GL[M > 0 ? M : 1], GM[NMID], WB;
    const int log_block = a.log_block < (N - 1) ? a.log_block : (N - 1);
    const uint64_t block_len = 1ull << log_block;
    const int mm = M < log_block ? M : log_block;   // chunk = 2^mm states
    bool aborted = false;

    for (uint64_t g0 = g_begin; g0 < g_end; g0 += block_len) {
        if (*a.abort_flag) { aborted = true; break; }
        // exact FP64 row sum at state g0
        df s;
        {
            const uint64_t gr = g0 ^ (g0 >> 1);
            double v = 0.0;
            if (live)
                for (int j = 0; j < N; j++) {
                    const double x = Ab[lane * N + j] * rscale;
                    v += (j < N - 1 && ((gr >> j) & 1)) ? -x : x;
                }
            s = live ? df_from(v) : df{1.f, 0.f};
        }
#pragma unroll
        for (int t = 0; t < (M > 0 ? M : 1); t++) GL[t] = df{0.f, 0.f};
#pragma unroll
        for (int t = 0; t < NMID; t++) GM[t] = df{0.f, 0.f};
        WB = df{0.f, 0.f};
        df fblk = df{0.f, 0.f};
        float fabs_blk = 0.f, gabs_blk = 0.f;
        for (uint64_t c0 = g0; c0 < g0 + block_len; c0 += (1ull << mm)) {
            df W = df{0.f, 0.f};
            df V[M > 0 ? M : 1];
#pragma unroll
            for (int t = 0; t < (M > 0 ? M : 1); t++) V[t] = df{0.f, 0.f};
#pragma unroll
            for (int r = 0; r < (1 << M); r++) {
                if (r >= (1 << mm)) break;
                const uint64_t g = c0 + r;
                if (g != g0) {
                    const int j = __ffsll((long long)g) - 1;
                    const bool sub = ((g >> (j + 1)) & 1) == 0;
                    const df d = tab[wib][j][lane];
                    if (live) s = df_add(s, sub ? df_neg(d) : d);
                }
                // butterfly: T = prod_l s_l.  The all-but-self products
                // E = prod_{l != lane} s_l (gradient only) are T / s_l, one
                // double-float division instead of five more products, unless
                // some row sum is zero or tiny (|s| < 2^-24: then T could
                // have lost what E keeps), where a second product butterfly
                // gives them directly.
                df T = s, E = df{1.f, 0.f};
#pragma unroll
                for (int lv = 0; lv < LEV; lv++) T = df_mul(T, df_shfl_xor(T, 1 << lv));
                if (GRAD) {
                    if (!__any_sync(0xffffffffu, fabsf(s.hi) < 5.9604645e-8f)) {
                        E = df_div(T, s);
                    } else {
                        df U = s;
#pragma unroll
                        for (int lv = 0; lv < LEV; lv++) {
                            const df o = df_shfl_xor(U, 1 << lv);
                            E = df_mul(E, o);
                            U = df_mul(U, o);
                        }
                    }
                }
                const bool odd = g & 1;                // Glynn sign (-1)^g
                const df term = odd ? df_neg(T) : T;
                fblk = df_add(fblk, term);
                fabs_blk += fabsf(T.hi);
                if (GRAD) {
                    const df w = odd ? df_neg(E) : E;
                    gabs_blk += fabsf(E.hi);
                    W = df_add(W, w);
#pragma unroll
                    for (int t = 0; t < M; t++) {
                        // sign of column t at g: bits t, t+1 of g; bit M
                        // (t = M-1) is applied per chunk below
                        const int bt = (r >> t) & 1;
                        const int bt1 = t + 1 < M ? ((r >> (t + 1)) & 1) : 0;
                        V[t] = df_add(V[t], (bt ^ bt1) ? df_neg(w) : w);
                    }
                }
            }
            if (GRAD) {
                const uint64_t gc = c0 ^ (c0 >> 1);
#pragma unroll
                for (int j = 0; j < M; j++) {
                    // column M-1 also depends on bit M of the chunk start
                    const bool flip = (j == M - 1) && ((c0 >> M) & 1);
                    GL[j] = df_add(GL[j], flip ? df_neg(V[j]) : V[j]);
                }
#pragma unroll
                for (int t = 0; t < NMID; t++) {
                    const int j = M + t;
                    if (j < N - 1 && j < log_block) {
                        const bool neg = (gc >> j) & 1;
                        GM[t] = df_add(GM[t], neg ? df_neg(W) : W);
                    }
                }
                WB = df_add(WB, W);
            }
        }
        kahan(fsum, fcomp, df_to(fblk));
        fabs_sum += (double)fabs_blk;
        gabs += (double)gabs_blk;
        if (GRAD && live) {
            // columns j >= log_block: the block's one sign (gray bit j of the
            // block start; the last column +)
            const uint64_t gb = g0 ^ (g0 >> 1);
            const double wb = df_to(WB);
#pragma unroll
            for (int j = 0; j < N; j++) {
                double v;
                if (j < M) {
                    v = df_to(GL[j]);
                } else if (j - M < NMID && j < N - 1 && j < log_block) {
                    v = df_to(GM[j - M < NMID ? j - M : 0]);
                } else {
                    v = (j < N - 1 && ((gb >> j) & 1)) ? -wb : wb;
                }
                double sm = slot[4 + lane * N + j], cp = slot[4 + N * N + lane * N + j];
                kahan(sm, cp, v);
                slot[4 + lane * N + j] = sm;
                slot[4 + N * N + lane * N + j] = cp;
            }
        }
    }
    if (lane == 0) {
        slot[0] = fsum;
        slot[1] = fcomp;
        slot[2] = fabs_sum;
    }
    if (live) slot[4 + 2 * N * N + lane] = gabs;
    if (aborted && lane == 0) atomicExch(a.status, 1);
}

// Reduce the 2^log_w slots of each matrix; undo the row scaling and 2^(n-1).
struct F64Reduce {
    const double *A;
    const double *slots;
    int batch, n, log_w, want_grad;
    double *per, *grad, *abs_sum, *grad_abs;   // device outputs (grad/grad_abs may be null)
};

__global__ void glynn_f64_reduce(F64Reduce r) {
    const int b = blockIdx.x;
    const int n = r.n;
    const int W = 1 << r.log_w;
    const int sd = f64_slot_doubles(n);
    const double *base = r.slots + (size_t)b * W * sd;
    const double *Ab = r.A + (size_t)b * n * n;
    // row exponents (recomputed exactly as in the walk kernel)
    __shared__ int ex[32];
    __shared__ int ex_total;
    if (threadIdx.x < n) {
        double rowsum = 0.0;
        for (int j = 0; j < n; j++) rowsum += fabs(Ab[threadIdx.x * n + j]);
        int e = 0;
        if (rowsum > 0.0) { frexp(rowsum, &e); e = -e; }
        ex[threadIdx.x] = e;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int i = 0; i < n; i++) t += ex[i];
        ex_total = t;
        double s = 0, c = 0, as = 0;
        for (int w = 0; w < W; w++) {
            kahan(s, c, base[(size_t)w * sd + 0]);
            kahan(s, c, -base[(size_t)w * sd + 1]);
            as += base[(size_t)w * sd + 2];
        }
        r.per[b] = ldexp(s, -t - (n - 1));
        if (r.abs_sum) r.abs_sum[b] = ldexp(as, -t - (n - 1));
    }
    __syncthreads();
    if (!r.want_grad) return;
    for (int ij = threadIdx.x; ij < n * n; ij += blockDim.x) {
        const int i = ij / n;
        double s = 0, c = 0;
        for (int w = 0; w < W; w++) {
            kahan(s, c, base[(size_t)w * sd + 4 + ij]);
            kahan(s, c, -base[(size_t)w * sd + 4 + n * n + ij]);
        }
        // E_i was formed from scaled rows l != i: undo 2^(sum_{l != i} e_l)
        r.grad[(size_t)b * n * n + ij] = ldexp(s, -(ex_total - ex[i]) - (n - 1));
    }
    if (r.grad_abs)
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double as = 0;
            for (int w = 0; w < W; w++) as += base[(size_t)w * sd + 4 + 2 * n * n + i];
            r.grad_abs[(size_t)b * n + i] = ldexp(as, -(ex_total - ex[i]) - (n - 1));
        }
}

template <int N>
static cudaError_t launch_f64(const F64Args &a, cudaStream_t s) {
    const long warps = (long)a.batch << a.log_w;
    if (a.want_grad)
        glynn_f64_kernel<N, true><<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(a);
    else
        glynn_f64_kernel<N, false><<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(a);
    return cudaGetLastError();
}

static cudaError_t launch_f64_any(int n, const F64Args &a, cudaStream_t s) {
    switch (n) {
#define PG_F64_CASE(NN) case NN: return launch_f64<NN>(a, s);
        PG_F64_CASE(2) PG_F64_CASE(3) PG_F64_CASE(4) PG_F64_CASE(5) PG_F64_CASE(6)
        PG_F64_CASE(7) PG_F64_CASE(8) PG_F64_CASE(9) PG_F64_CASE(10) PG_F64_CASE(11)
        PG_F64_CASE(12) PG_F64_CASE(13) PG_F64_CASE(14) PG_F64_CASE(15) PG_F64_CASE(16)
        PG_F64_CASE(17) PG_F64_CASE(18) PG_F64_CASE(19) PG_F64_CASE(20) PG_F64_CASE(21)
        PG_F64_CASE(22) PG_F64_CASE(23) PG_F64_CASE(24) PG_F64_CASE(25) PG_F64_CASE(26)
        PG_F64_CASE(27) PG_F64_CASE(28) PG_F64_CASE(29) PG_F64_CASE(30) PG_F64_CASE(31)
        PG_F64_CASE(32)
#undef PG_F64_CASE
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace pg

extern "C" int pg_glynn_f64_dev(const double *A, int batch, int n, double *per, double *grad,
                                double *abs_sum, double *grad_abs, void *stream) {
    using namespace pg;
    if (batch < 0 || n < 0 || n > 63) return fail(PG_ERANGE, "FP64 engine supports 0 <= n <= 63");
    if (batch == 0) return PG_OK;
    if (!A || !per) return fail(PG_EINVAL, "null argument");
    if (n <= 1) return fail(PG_ERANGE, "orders 0 and 1 are handled by the caller");
    if (n > 32) {
        // orders 33..63: forward only, two rows per lane (f64_wide.cuh)
        if (grad || grad_abs)
            return fail(PG_ERANGE, "the FP64 gradient supports n <= 32 (forward up to 63)");
        return glynn_wide_run(A, nullptr, batch, n, 0, 1ull << (n - 1), true, per, nullptr,
                              abs_sum, (cudaStream_t)stream);
    }
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    // warps per matrix: about four resident waves overall (~20 resident
    // warps per SM at this kernel's register use) so the equal-work warps
    // leave a small tail, but >= 2^12 states per warp (the exact
    // re-initialisation period)
    const int log_states = n - 1;
    int log_w = 0;
    while ((((long)batch << log_w) < (long)dev.sm_count * 80) &&
           log_states - (log_w + 1) >= 12)
        log_w++;
    const int log_block = std::min(12, log_states - log_w);
    const size_t slots = (size_t)batch << log_w;
    const size_t bytes = slots * f64_slot_doubles(n) * sizeof(double) + 256;
    Workspace *ws;
    st = workspace(&ws, bytes, 64);
    if (st != PG_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : ws->stream;
    double *slot_mem = (double *)ws->dev;
    int *status = (int *)((char *)ws->dev + bytes - 256);
    PG_CUDA(cudaMemsetAsync(ws->dev, 0, bytes, s));
    F64Args a;
    a.A = A;
    a.batch = batch;
    a.n = n;
    a.log_w = log_w;
    a.log_block = log_block;
    a.want_grad = grad != nullptr;
    a.slots = slot_mem;
    a.abort_flag = abort_dev;
    a.status = status;
    PG_CUDA(launch_f64_any(n, a, s));
    F64Reduce r;
    r.A = A;
    r.slots = slot_mem;
    r.batch = batch;
    r.n = n;
    r.log_w = log_w;
    r.want_grad = grad != nullptr;
    r.per = per;
    r.grad = grad;
    r.abs_sum = abs_sum;
    r.grad_abs = grad_abs;
    glynn_f64_reduce<<<batch, 256, 0, s>>>(r);
    PG_CUDA(cudaGetLastError());
    int hstatus = 0;
    PG_CUDA(cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    if (hstatus) return fail(PG_EABORT, "FP64 launch aborted by pg_abort()");
    return PG_OK;
}

// ---------------------------------------------------------------------------
// Complex FP64 Glynn permanent (forward), double-float complex arithmetic.
// Same walk as glynn_f64_kernel (lane = row, shuffle butterfly for the row
// product, exact FP64 re-initialisation every 2^log_block states, Kahan FP64
// flushes into per-warp slots); complex counterpart of rivin-perm
// permanent_glynn_kernel<true> (perm_parallel_cuda.cu:68-209).
namespace pg {

struct C64Args {
    const double *Are, *Aim;   // [batch][n][n]
    int batch, log_w, log_block;
    double *slots;             // [batch << log_w][8]: re sum/comp, im sum/comp, abs
    volatile const int *abort_flag;
    int *status;
};

template <int N>
__global__ void __launch_bounds__(128) glynn_c64_kernel(C64Args a) {
    constexpr int LEV = N <= 2 ? 1 : N <= 4 ? 2 : N <= 8 ? 3 : N <= 16 ? 4 : 5;
    __shared__ dc tab[4][N - 1][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const long gw = (long)blockIdx.x * 4 + wib;
    if (gw >= ((long)a.batch << a.log_w)) return;
    const int b = (int)(gw >> a.log_w);
    const uint64_t part = (uint64_t)(gw & ((1 << a.log_w) - 1));
    const uint64_t per_warp = (1ull << (N - 1)) >> a.log_w;
    const uint64_t g_begin = part * per_warp, g_end = g_begin + per_warp;
    const double *Ar = a.Are + (size_t)b * N * N, *Ai = a.Aim + (size_t)b * N * N;
    const bool live = lane < N;
    // power-of-two row scaling by the row's sum of |re| + |im|
    double rowsum = 0.0;
    if (live)
        for (int j = 0; j < N; j++) rowsum += fabs(Ar[lane * N + j]) + fabs(Ai[lane * N + j]);
    int ex = 0;
    if (live && rowsum > 0.0) { frexp(rowsum, &ex); ex = -ex; }
    const double rs = ldexp(1.0, ex);
    for (int j = 0; j < N - 1; j++)
        tab[wib][j][lane] = live ? dc{df_from(2.0 * Ar[lane * N + j] * rs),
                                      df_from(2.0 * Ai[lane * N + j] * rs)}
                                 : dc{{0.f, 0.f}, {0.f, 0.f}};
    __syncwarp();
    double sre = 0, cre = 0, sim = 0, cim = 0, asum = 0;
    const int log_block = a.log_block < (N - 1) ? a.log_block : (N - 1);
    const uint64_t block_len = 1ull << log_block;
    bool aborted = false;
    for (uint64_t g0 = g_begin; g0 < g_end; g0 += block_len) {
        if (*a.abort_flag) { aborted = true; break; }
        dc s;
        {
            const uint64_t gr = g0 ^ (g0 >> 1);
            double vr = 0, vi = 0;
            if (live)
                for (int j = 0; j < N; j++) {
                    const bool neg = j < N - 1 && ((gr >> j) & 1);
                    vr += neg ? -Ar[lane * N + j] * rs : Ar[lane * N + j] * rs;
                    vi += neg ? -Ai[lane * N + j] * rs : Ai[lane * N + j] * rs;
                }
            s = live ? dc{df_from(vr), df_from(vi)} : dc{{1.f, 0.f}, {0.f, 0.f}};
        }
        dc blk = dc{{0.f, 0.f}, {0.f, 0.f}};
        float blk_abs = 0.f;
        for (uint64_t g = g0; g < g0 + block_len; g++) {
            if (g != g0) {
                const int j = __ffsll((long long)g) - 1;
                const bool sub = ((g >> (j + 1)) & 1) == 0;
                const dc d = tab[wib][j][lane];
                if (live) {
                    s.re = df_add(s.re, sub ? df_neg(d.re) : d.re);
                    s.im = df_add(s.im, sub ? df_neg(d.im) : d.im);
                }
            }
            dc T = s;
#pragma unroll
            for (int lv = 0; lv < LEV; lv++) {
                const dc o = dc{df_shfl_xor(T.re, 1 << lv), df_shfl_xor(T.im, 1 << lv)};
                T = dc_mul(T, o);
            }
            if (g & 1) { T.re = df_neg(T.re); T.im = df_neg(T.im); }
            blk.re = df_add(blk.re, T.re);
            blk.im = df_add(blk.im, T.im);
            blk_abs += hypotf(T.re.hi, T.im.hi);
        }
        kahan(sre, cre, df_to(blk.re));
        kahan(sim, cim, df_to(blk.im));
        asum += (double)blk_abs;
    }
    if (lane == 0) {
        double *slot = a.slots + (size_t)gw * 8;
        slot[0] = sre; slot[1] = cre; slot[2] = sim; slot[3] = cim; slot[4] = asum;
        if (aborted) atomicExch(a.status, 1);
    }
}

__global__ void glynn_c64_reduce(const double *Are, const double *Aim, const double *slots,
                                 int n, int log_w, double *per_re, double *per_im,
                                 double *abs_sum) {
    const int b = blockIdx.x;
    if (threadIdx.x != 0) return;
    int et = 0;
    for (int i = 0; i < n; i++) {
        double rowsum = 0.0;
        for (int j = 0; j < n; j++)
            rowsum += fabs(Are[(size_t)b * n * n + i * n + j]) + fabs(Aim[(size_t)b * n * n + i * n + j]);
        int e = 0;
        if (rowsum > 0.0) { frexp(rowsum, &e); e = -e; }
        et += e;
    }
    double sr = 0, cr = 0, si = 0, ci = 0, as = 0;
    for (int w = 0; w < (1 << log_w); w++) {
        const double *sl = slots + ((size_t)b * (1 << log_w) + w) * 8;
        kahan(sr, cr, sl[0]); kahan(sr, cr, -sl[1]);
        kahan(si, ci, sl[2]); kahan(si, ci, -sl[3]);
        as += sl[4];
    }
    per_re[b] = ldexp(sr, -et - (n - 1));
    per_im[b] = ldexp(si, -et - (n - 1));
    if (abs_sum) abs_sum[b] = ldexp(as, -et - (n - 1));
}

static cudaError_t launch_c64_any(int n, const C64Args &a, cudaStream_t s) {
    const long warps = (long)a.batch << a.log_w;
    const unsigned grid = (unsigned)((warps + 3) / 4);
    switch (n) {
#define PG_C64_CASE(NN) case NN: glynn_c64_kernel<NN><<<grid, 128, 0, s>>>(a); break;
        PG_C64_CASE(2) PG_C64_CASE(3) PG_C64_CASE(4) PG_C64_CASE(5) PG_C64_CASE(6)
        PG_C64_CASE(7) PG_C64_CASE(8) PG_C64_CASE(9) PG_C64_CASE(10) PG_C64_CASE(11)
        PG_C64_CASE(12) PG_C64_CASE(13) PG_C64_CASE(14) PG_C64_CASE(15) PG_C64_CASE(16)
        PG_C64_CASE(17) PG_C64_CASE(18) PG_C64_CASE(19) PG_C64_CASE(20) PG_C64_CASE(21)
        PG_C64_CASE(22) PG_C64_CASE(23) PG_C64_CASE(24) PG_C64_CASE(25) PG_C64_CASE(26)
        PG_C64_CASE(27) PG_C64_CASE(28) PG_C64_CASE(29) PG_C64_CASE(30) PG_C64_CASE(31)
        PG_C64_CASE(32)
#undef PG_C64_CASE
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace pg

extern "C" int pg_glynn_c64_dev(const double *Are, const double *Aim, int batch, int n,
                                double *per_re, double *per_im, double *abs_sum, void *stream) {
    using namespace pg;
    if (batch < 0 || n < 2 || n > 63) return fail(PG_ERANGE, "complex FP64 engine supports 2 <= n <= 63");
    if (batch == 0) return PG_OK;
    if (!Are || !Aim || !per_re || !per_im) return fail(PG_EINVAL, "null argument");
    if (n > 32)   // two rows per lane (f64_wide.cuh)
        return glynn_wide_run(Are, Aim, batch, n, 0, 1ull << (n - 1), true, per_re, per_im,
                              abs_sum, (cudaStream_t)stream);
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    const int log_states = n - 1;
    int log_w = 0;
    while ((((long)batch << log_w) < (long)dev.sm_count * 80) && log_states - (log_w + 1) >= 12)
        log_w++;
    const size_t bytes = ((size_t)batch << log_w) * 8 * sizeof(double) + 256;
    Workspace *ws;
    st = workspace(&ws, bytes, 64);
    if (st != PG_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : ws->stream;
    int *status = (int *)((char *)ws->dev + bytes - 256);
    PG_CUDA(cudaMemsetAsync(ws->dev, 0, bytes, s));
    C64Args a;
    a.Are = Are; a.Aim = Aim; a.batch = batch; a.log_w = log_w;
    a.log_block = std::min(12, log_states - log_w);
    a.slots = (double *)ws->dev;
    a.abort_flag = abort_dev;
    a.status = status;
    PG_CUDA(launch_c64_any(n, a, s));
    glynn_c64_reduce<<<batch, 32, 0, s>>>(Are, Aim, (const double *)ws->dev, n, log_w,
                                          per_re, per_im, abs_sum);
    PG_CUDA(cudaGetLastError());
    int hstatus = 0;
    PG_CUDA(cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    if (hstatus) return fail(PG_EABORT, "complex FP64 launch aborted by pg_abort()");
    return PG_OK;
}

// Host-pointer form of pg_glynn_f64_dev for callers without device memory of
// their own (ctypes users, other languages' FFIs): device buffers for the
// call are allocated here (the library's workspace is the kernel's own
// scratch), the results are copied back and the buffers freed.
extern "C" int pg_glynn_f64_fwd_bwd(const double *A, int batch, int n, double *per,
                                    double *grad, double *abs_sum) {
    using namespace pg;
    if (batch < 0 || n < 0 || n > 63) return fail(PG_ERANGE, "FP64 engine supports 0 <= n <= 63");
    if (batch == 0) return PG_OK;
    if (!per || (n > 0 && !A)) return fail(PG_EINVAL, "null argument");
    if (n > 32 && grad)
        return fail(PG_ERANGE, "the FP64 gradient supports n <= 32 (forward up to 63)");
    if (n <= 1) {
        for (int b = 0; b < batch; b++) {
            per[b] = n == 0 ? 1.0 : A[b];
            if (grad && n == 1) grad[b] = 1.0;
            if (abs_sum) abs_sum[b] = n == 0 ? 1.0 : std::fabs(A[b]);
        }
        return PG_OK;
    }
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    const size_t na = (size_t)batch * n * n;
    const size_t bytes = (na + (grad ? na : 0) + 2 * (size_t)batch) * sizeof(double);
    double *d = nullptr;
    PG_CUDA(cudaMalloc(&d, bytes));
    double *dA = d, *dgrad = grad ? d + na : nullptr;
    double *dper = d + na + (grad ? na : 0), *dabs = dper + batch;
    cudaError_t e = cudaMemcpy(dA, A, na * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "cudaMemcpy(A)");
    }
    st = pg_glynn_f64_dev(dA, batch, n, dper, dgrad, dabs, nullptr, nullptr);
    if (st == PG_OK) {
        e = cudaMemcpy(per, dper, (size_t)batch * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && grad)
            e = cudaMemcpy(grad, dgrad, na * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && abs_sum)
            e = cudaMemcpy(abs_sum, dabs, (size_t)batch * sizeof(double), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpy(results)");
    }
    cudaFree(d);
    return st;
}

// pg_glynn_c64_dev with host pointers: the real and imaginary planes
// [batch][n][n] in, per_re/per_im[batch] and abs_sum[batch] (nullable)
// out; 0 <= n <= 63 (n <= 1 on the host).  Device buffers for the call are
// allocated and freed inside.  Replaces permanent_parallel_complex
// (perm_parallel_cuda.cu:416-498), host planes in and host values out.
extern "C" int pg_glynn_c64(const double *Are, const double *Aim, int batch, int n,
                            double *per_re, double *per_im, double *abs_sum) {
    using namespace pg;
    if (batch < 0 || n < 0 || n > 63)
        return fail(PG_ERANGE, "complex FP64 engine supports 0 <= n <= 63");
    if (batch == 0) return PG_OK;
    if (!per_re || !per_im || (n > 0 && (!Are || !Aim))) return fail(PG_EINVAL, "null argument");
    if (n <= 1) {
        for (int b = 0; b < batch; b++) {
            per_re[b] = n == 0 ? 1.0 : Are[b];
            per_im[b] = n == 0 ? 0.0 : Aim[b];
            if (abs_sum) abs_sum[b] = n == 0 ? 1.0 : std::hypot(Are[b], Aim[b]);
        }
        return PG_OK;
    }
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    const size_t na = (size_t)batch * n * n;
    const size_t bytes = (2 * na + 3 * (size_t)batch) * sizeof(double);
    double *d = nullptr;
    PG_CUDA(cudaMalloc(&d, bytes));
    double *dre = d, *dim = d + na, *dpre = d + 2 * na, *dpim = dpre + batch,
           *dabs = dpim + batch;
    cudaError_t e = cudaMemcpy(dre, Are, na * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dim, Aim, na * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "cudaMemcpy(A)");
    }
    st = pg_glynn_c64_dev(dre, dim, batch, n, dpre, dpim, dabs, nullptr);
    if (st == PG_OK) {
        e = cudaMemcpy(per_re, dpre, (size_t)batch * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(per_im, dpim, (size_t)batch * sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && abs_sum)
            e = cudaMemcpy(abs_sum, dabs, (size_t)batch * sizeof(double), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpy(results)");
    }
    cudaFree(d);
    return st;
}
