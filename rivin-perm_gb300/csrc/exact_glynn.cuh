// Exact Glynn kernel: no moduli at all.
//
// For integer matrices whose row-sum bound B_i = sum_j |a_ij| is small (every
// benchmark matrix: entries in [-8,8] give B_i <= 8n), the Glynn row sums
// s_i(d) = sum_j d_j a_ij fit in int32 and every term prod_i s_i is an exact
// integer of at most sum_i log2(B_i) bits.  This kernel keeps the row sums
// exact, multiplies them in groups of G rows with plain 32-bit IMUL (the host
// permutes rows so that every group's bound product is < 2^31), folds the
// term's sign into the first group, forms the signed product of the first
// NG-1 groups as a multi-word integer (mul.wide products plus an ALU carry
// chain), and multiplies it by the last group into 64-bit column
// accumulators that are added into an NL-word two's-complement accumulator
// every 2^LOGU terms (col_acc.cuh).
//
// Versus a CRT residue walk this removes the modular reductions and the
// per-prime repetition: for n = 32, entries in [-8,8], one exact term costs
// 24 IMUL + 28 mul.wide, while 8 CRT primes cost 8 * 31 Montgomery
// products (~750 IMAD-class instructions) plus 8 * 32 modular row updates.
//
// Traversal, sign and chunking follow the residue walk of rivin-perm
// perm_c_omp.c:556-639: states in Gray order with the last column's sign
// fixed, Glynn sign (-1)^g.  Chunks of 2^log_len states are aligned, so at
// local step i every lane of a warp toggles column ctz(i) and reads the same
// table row (shared-memory broadcast).  A thread walks a contiguous range of
// chunks; crossing a chunk boundary is an ordinary Gray step.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "col_acc.cuh"

#ifndef EXACT_LOGU
#define EXACT_LOGU 2
#endif
#ifndef EXACT_MIN_BLOCKS
#define EXACT_MIN_BLOCKS 0
#endif

namespace pg {

__device__ __forceinline__ constexpr int exact_ctz_small(int r) {
    return (r & 1) ? 0 : (r & 2) ? 1 : (r & 4) ? 2 : (r & 8) ? 3 : 4;
}

template <int N, int G>
struct ExactShape {
    static constexpr int NP = (N + 3) & ~3;
    static constexpr int NG = (N + G - 1) / G;           // product words
    static constexpr int NL = NG + (N > 32 ? 2 : 1);     // accumulator words
    static constexpr int LOGU = (N - 1) < EXACT_LOGU ? (N - 1) : EXACT_LOGU;
    static constexpr int NR = NG > 1 ? NG - 1 : 1;       // words of the leading product
};

// Float rows (FR > 0): in every group the first min(FR, size - 1) row sums
// are kept as exact FP32 values (the host orders each group by bound and
// checks |s| < 2^24 and a bound product below 2^22 for them).  Their
// product is formed by FMULs on the otherwise idle FP32 pipes, made an
// integer by adding 1.5 * 2^23 (the low mantissa bits of the sum are then
// the integer plus 2^22) and finished by IMULs with the group's integer
// rows: for groups of 4 with 3 float rows one IMAD-pipe instruction per
// group instead of three.  Table entries and initial sums of the float rows
// hold FP32 bit patterns.  The compiled shapes are listed in exact_frows.cu.
__host__ __device__ constexpr int exact_group_size(int N, int G, int g) {
    return N - g * G < G ? N - g * G : G;
}
__host__ __device__ constexpr int exact_float_rows(int N, int G, int FR, int g) {
    return FR <= 0 ? 0 : FR < exact_group_size(N, G, g) - 1 ? FR : exact_group_size(N, G, g) - 1;
}
__host__ __device__ constexpr bool exact_float_row(int N, int G, int FR, int i) {
    return i % G < exact_float_rows(N, G, FR, i / G);
}

template <int N, int G, int FR>
__device__ __forceinline__ int32_t exact_row_add(int i, int32_t s, int32_t d) {
    if (exact_float_row(N, G, FR, i)) return __float_as_int(__int_as_float(s) + __int_as_float(d));
    return s + d;
}

// Row sums of Gray state `start`: init - sum_{j in gray(start)} 2 a_j.
template <int N, int G = 1, int FR = 0>
__device__ __forceinline__ void exact_init(const int32_t *tab, const int32_t *init,
                                           int32_t *s, uint64_t start) {
    constexpr int NP = (N + 3) & ~3;
    const uint64_t gs = start ^ (start >> 1);
#pragma unroll
    for (int i = 0; i < N; i++) s[i] = init[i];
    for (int j = 0; j < N - 1; j++) {
        if ((gs >> j) & 1) {
            const int32_t *col = tab + (2 * j + 1) * NP;
#pragma unroll
            for (int i = 0; i < N; i++) s[i] = exact_row_add<N, G, FR>(i, s[i], col[i]);
        }
    }
}

// Column form of one term: the sign and the first NG-1 group products give
// the signed NR-word R, the last group's magnitude y multiplies R into the
// columns (first: the columns start from this term).  For NG == 1, R = +-1.
// R[0..K-1] (signed) *= |x[K]| ... |x[END-1]|, one word per factor.
template <int K, int END>
struct ProdChainS {
    static __device__ __forceinline__ void run(uint32_t *R, const int32_t *x) {
        MulWordS<K>::apply(R, (uint32_t)abs(x[K]));
        ProdChainS<K + 1, END>::run(R, x);
    }
};
template <int END>
struct ProdChainS<END, END> {
    static __device__ __forceinline__ void run(uint32_t *, const int32_t *) {}
};

template <int N, int G, int FR = 0>
__device__ __forceinline__ void exact_term_col(const int32_t *s, uint64_t *col, int64_t &colt,
                                               uint32_t odd, bool first) {
    using S = ExactShape<N, G>;
    constexpr int NG = S::NG, NR = S::NR;
    int32_t x[NG];
#pragma unroll
    for (int g = 0; g < NG; g++) {
        const int nf = exact_float_rows(N, G, FR, g), sz = exact_group_size(N, G, g);
        if (nf > 0) {
            float t = __int_as_float(s[g * G]);
#pragma unroll
            for (int u = 1; u < G; u++)
                if (u < nf) t *= __int_as_float(s[g * G + u]);
            x[g] = __float_as_int(t + 12582912.0f) - 0x4B400000;
#pragma unroll
            for (int u = 1; u < G; u++)
                if (u >= nf && u < sz) x[g] *= s[g * G + u];
        } else {
            x[g] = s[g * G];
#pragma unroll
            for (int t = 1; t < G; t++)
                if (g * G + t < N) x[g] *= s[g * G + t];
        }
    }
    uint32_t sx = odd << 31;
#pragma unroll
    for (int g = (NG > 1 ? 1 : 0); g < NG; g++) sx ^= (uint32_t)x[g];
    const int32_t m = (int32_t)sx >> 31;
    uint32_t R[NR + 1];
    R[0] = (uint32_t)(((NG > 1 ? x[0] : 1) ^ m) - m);
    ProdChainS<1, (NG > 1 ? NG - 1 : 1)>::run(R, x);
    const uint32_t y = (uint32_t)abs(x[NG - 1]);
#pragma unroll
    for (int l = 0; l < NR - 1; l++) {
        const uint64_t p = (uint64_t)R[l] * y;
        col[l] = first ? p : col[l] + p;
    }
    const int64_t pt = (int64_t)(int32_t)R[NR - 1] * (int64_t)y;
    colt = first ? pt : colt + pt;
}

// Walk chunks [c_begin, c_end) (row sums s already at state c_begin*2^log_len)
// adding every term into acc.  Returns false if the abort word was seen.
template <int N, int G, int FR = 0>
__device__ __forceinline__ bool exact_walk(const int32_t *tab, int32_t *s, uint32_t *acc,
                                           uint64_t c_begin, uint64_t c_end, int log_len,
                                           volatile const int *abort_flag) {
    using S = ExactShape<N, G>;
    constexpr int NP = S::NP, LOGU = S::LOGU, U = 1 << LOGU;
    const uint32_t Q = (1u << log_len) >> LOGU;
    uint64_t col[S::NR > 1 ? S::NR - 1 : 1];
    int64_t colt;
    // the host-mapped abort word is read once per 2^16 states (per chunk for
    // longer chunks), from the thread's second period on: threads of a short
    // launch never read it, so thousands of warps do not queue on one
    // host-memory word before their work starts
    const uint64_t poll = log_len >= 16 ? 0 : (1ull << (16 - log_len)) - 1;
    for (uint64_t c = c_begin; c < c_end; c++) {
        if (c != c_begin && ((c - c_begin) & poll) == 0 && *abort_flag) return false;
        const uint32_t hib = (uint32_t)(c & 1) << log_len;
        for (uint32_t q = 0; q < Q; q++) {
            const uint32_t g32 = (q << LOGU) | hib;
#pragma unroll
            for (int r = 0; r < U; r++) {
                bool step = true;
                int j, sub;
                if (r != 0) {
                    j = exact_ctz_small(r);
                    if (j + 1 < LOGU) sub = ((r >> (j + 1)) & 1) == 0;
                    else sub = ((g32 >> LOGU) & 1) == 0;
                } else if (q != 0) {
                    j = __ffs(q) - 1 + LOGU;
                    sub = ((g32 >> (j + 1)) & 1) == 0;
                } else {
                    // chunk boundary g = c * 2^log_len (lanes may differ here)
                    step = c != c_begin;
                    const int jc = __ffsll((long long)c) - 1;
                    j = log_len + jc;
                    sub = ((c >> (jc + 1)) & 1) == 0;
                }
                if (step) {
                    const int4 *col =
                        reinterpret_cast<const int4 *>(tab + (2 * j + sub) * NP);
#pragma unroll
                    for (int v = 0; v < NP / 4; v++) {
                        const int4 d = col[v];
                        if (4 * v + 0 < N) s[4 * v + 0] = exact_row_add<N, G, FR>(4 * v + 0, s[4 * v + 0], d.x);
                        if (4 * v + 1 < N) s[4 * v + 1] = exact_row_add<N, G, FR>(4 * v + 1, s[4 * v + 1], d.y);
                        if (4 * v + 2 < N) s[4 * v + 2] = exact_row_add<N, G, FR>(4 * v + 2, s[4 * v + 2], d.z);
                        if (4 * v + 3 < N) s[4 * v + 3] = exact_row_add<N, G, FR>(4 * v + 3, s[4 * v + 3], d.w);
                    }
                }
                // chunks start at even states, so (-1)^g = (-1)^r
                exact_term_col<N, G, FR>(s, col, colt, (uint32_t)(r & 1), r == 0);
            }
            FoldCols<S::NR, S::NL>::apply(acc, col, colt);
        }
    }
    return true;
}

struct ExactArgs {
    const int32_t *tab;        // [N-1][2][NP]  +2a_ij (dir 0) / -2a_ij (dir 1)
    const int32_t *init;       // [NP] row sums of the all-plus state
    unsigned long long *acc;   // [NL] per-word sums (two's complement, zeroed)
    int *status;
    // Per-block word slots [NL][gridDim] (written in full by every launch),
    // or nullptr: blocks then add their words into acc with atomics.  The
    // finishing kernel (exact_finish) turns either into the result words.
    unsigned long long *part = nullptr;
    volatile const int *abort_flag;
    uint64_t chunks;           // chunks to walk: [chunk0, chunk0 + chunks)
    int log_len;               // >= LOGU, <= 30
    uint64_t chunk0;           // first chunk (0 for a whole traversal)
    int threads = 256;         // threads per block: a multiple of 32, <= 256
};

// Launch shape for a walk of 2^log_states states: one resident wave of
// `occ` 256-thread blocks per SM while every thread still gets at least
// EXACT_MIN_THREAD_STATES states; shorter walks put the same number of
// whole warps on every SM (smaller blocks) instead of idling SMs.  Chunks
// are sized for ~128 per thread on long walks and go down to
// 2^EXACT_MIN_CHUNK_LOG states on short ones (the boundary step is the only
// one whose column differs between lanes).
#ifndef EXACT_MIN_THREAD_STATES
#define EXACT_MIN_THREAD_STATES 64
#endif
#ifndef EXACT_MIN_CHUNK_LOG
#define EXACT_MIN_CHUNK_LOG 2
#endif
void exact_launch_shape(int log_states, int occ, int sm_count, uint64_t *blocks,
                        int *threads, int *log_len);

// Resident blocks per SM requested from ptxas: a register budget of about
// N + 64 per thread (row sums plus the product/accumulator words) measured
// fastest; tighter budgets spill.
__host__ __device__ constexpr int exact_min_blocks(int N) {
    return EXACT_MIN_BLOCKS > 0 ? EXACT_MIN_BLOCKS
           : (65536 / (256 * (N + 64))) < 1 ? 1
           : (65536 / (256 * (N + 64))) > 4 ? 4
           : (65536 / (256 * (N + 64)));
}

// Epilogue of the exact kernels, after the warps' word sums are in red[][]
// and the block has synchronised: the block's words go to its own slot of
// part[] (no two blocks touch one address), or with part == nullptr are
// added into acc[] with atomics; an abort is recorded in *status.  Summing
// the slots is left to a one-block kernel launched after it (exact_finish):
// doing it in the last block to finish made the compiler lay out the walk
// loop worse (1-3 % at orders 28..32).
template <int NL>
__device__ __forceinline__ void exact_epilogue(long long (*red)[NL], bool any_abort,
                                               unsigned long long *acc, unsigned long long *part,
                                               int *status) {
    if (threadIdx.x < NL) {
        long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w][threadIdx.x];
        if (part) part[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = (unsigned long long)t;
        else atomicAdd(acc + threadIdx.x, (unsigned long long)t);
    }
    if (threadIdx.x == 0 && any_abort) atomicExch(status, 1);
}

// Programmatic dependent launch of the finishing kernel: with
// EXACT_FINISH_PDL the walk kernels signal at their start that the
// dependent grid may be scheduled, the finishing kernel is launched with
// programmatic stream serialisation and its block waits (griddepcontrol.wait)
// until the walk grid has completed and its writes are visible.  The
// dependent grid is scheduled only after every walk block has started, so
// it never takes a slot a walk block is waiting for; its launch latency
// overlaps the walk instead of following it.
#ifndef EXACT_FINISH_PDL
#define EXACT_FINISH_PDL 1
#endif
__device__ __forceinline__ void exact_allow_dependents() {
#if EXACT_FINISH_PDL
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// Launches the finishing kernel on `stream` after an exact or 0/1 kernel of
// `blocks` blocks: out[0..nl) = the sum of the slots (or acc, re-zeroed,
// when part is nullptr), out[nl] = *status, then *status = 0 and, when
// given, *counter = 0 (the 0/1 kernel's chunk-group counter), so the next
// launch starts clean without a memset (pg_exact.cu).
cudaError_t exact_finish(const unsigned long long *part, int blocks, int nl,
                         unsigned long long *acc, int *status, unsigned long long *out,
                         cudaStream_t stream, unsigned long long *counter = nullptr);

template <int N, int G, int FR = 0>
__global__ void __launch_bounds__(256, exact_min_blocks(N))
exact_glynn_kernel(ExactArgs a) {
    using S = ExactShape<N, G>;
    constexpr int NP = S::NP, NL = S::NL, NCOL = N - 1;
    extern __shared__ int4 esmem[];
    int32_t *tab = reinterpret_cast<int32_t *>(esmem);
    exact_allow_dependents();
    for (int i = threadIdx.x; i < NCOL * 2 * NP / 4; i += blockDim.x)
        esmem[i] = reinterpret_cast<const int4 *>(a.tab)[i];
    __syncthreads();

    uint32_t acc[NL];
#pragma unroll
    for (int l = 0; l < NL; l++) acc[l] = 0;

    // one contiguous, balanced range of chunks per thread
    const uint64_t T = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t c_begin = a.chunk0 + tid * a.chunks / T;
    const uint64_t c_end = a.chunk0 + (tid + 1) * a.chunks / T;
    bool aborted = false;
    if (c_begin < c_end) {
        int32_t s[N];
        exact_init<N, G, FR>(tab, a.init, s, c_begin << a.log_len);
        aborted = !exact_walk<N, G, FR>(tab, s, acc, c_begin, c_end, a.log_len, a.abort_flag);
    }

    // Block reduction: word l < NL-1 contributes acc[l] (unsigned), the top
    // word is signed.  Sums of 64-bit words stay exact (< 2^54 in magnitude).
    __shared__ long long red[8][NL];
    __shared__ int any_abort;
    if (threadIdx.x == 0) any_abort = 0;
    __syncthreads();
    if (aborted) any_abort = 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int l = 0; l < NL; l++) {
        long long v = (l == NL - 1) ? (long long)(int32_t)acc[l] : (long long)acc[l];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp][l] = v;
    }
    __syncthreads();
    exact_epilogue<NL>(red, any_abort, a.acc, a.part, a.status);
}

template <int N, int G, int FR = 0>
cudaError_t launch_exact_glynn(const ExactArgs &args, int blocks,
                               cudaStream_t stream) {
    constexpr int NP = ExactShape<N, G>::NP;
    const size_t smem = (size_t)(N - 1) * 2 * NP * sizeof(int32_t);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(
            exact_glynn_kernel<N, G, FR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
            (int)smem);
        if (e != cudaSuccess) return e;
    }
    exact_glynn_kernel<N, G, FR><<<blocks, args.threads, smem, stream>>>(args);
    return cudaGetLastError();
}

template <int N, int G, int FR = 0>
int occupancy_exact_glynn() {
    constexpr int NP = ExactShape<N, G>::NP;
    const size_t smem = (size_t)(N - 1) * 2 * NP * sizeof(int32_t);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(exact_glynn_kernel<N, G, FR>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, exact_glynn_kernel<N, G, FR>,
                                                      256, smem) != cudaSuccess)
        return 1;
    return nb < 1 ? 1 : nb;
}

// Largest compiled group size (gen_exact_inst.py); hosts try G from here down.
constexpr int EXACT_MAX_G = 10;

// Float-row form (exact_float_row): 1 lets the host take it for the shapes
// exact_frows.cu compiles when a matrix's bounds allow.
#ifndef EXACT_FROWS
#define EXACT_FROWS 1
#endif

// Largest compiled float-row count for (N, G), 0 when none (exact_frows.cu).
int exact_frows_max(int N, int G);
// Orders each row group of `order` (n rows, groups of G) by increasing bound
// and checks that its first exact_float_rows(n, G, FR, g) rows qualify as
// float rows (bounds below 2^24, product below 2^22); on success rewrites
// `order` (same group membership) and returns true (pg_exact.cu).
bool exact_frows_arrange(const int64_t *A, int n, int G, int FR, int *order);
__host__ __device__ inline uint32_t exact_float_bits(float f) {
    union { float f; uint32_t u; } v;
    v.f = f;
    return v.u;
}
cudaError_t launch_exact_frows(int N, int G, int FR, const ExactArgs &args, int blocks,
                               cudaStream_t stream);
int occupancy_exact_frows(int N, int G, int FR);

// Compiled (N, G) pairs; returns cudaErrorInvalidValue / 0 when absent.
cudaError_t launch_exact_any(int N, int G, const ExactArgs &args, int blocks,
                             cudaStream_t stream);
int occupancy_exact_any(int N, int G);
bool exact_compiled(int N, int G);

// Largest bound product of the last row group: its magnitude multiplies
// each word of the running product into a 64-bit column 2^EXACT_LOGU times
// between folds.
constexpr uint64_t EXACT_LAST_GROUP_MAX = 1ull << (32 - EXACT_LOGU);

// Row order for group size G (rows [g*G, min((g+1)*G, n)) form group g) in
// which every group's product of row bounds B is < 2^31 and the last
// group's is <= EXACT_LAST_GROUP_MAX; n <= 48.  False if none was found.
bool exact_group_rows(const uint64_t *B, int n, int G, int *order);

}  // namespace pg
