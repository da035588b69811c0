// Exact Glynn kernel for 0/1 matrices: bit-sliced zero-row tracking and
// warp-compacted exact evaluation of the states that survive it.
//
// For a 0/1 matrix the Glynn row sum of state d is s_r = deg_r - 2 m_r,
// where m_r counts the row's ones in columns whose sign is minus.  A term
// is zero as soon as one row sum is zero, which needs an even degree and
// m_r = deg_r / 2; for the benchmark matrices that is most states
// (40 x 40 Bernoulli(1/2): ~92 %; the 4x4x5 grid: ~99.9 %).  The reference
// keeps int16 row sums, a zero counter and a ratio-updated product mod p
// for every state (perm_binary_omp.c:236-347, perm_binary_cuda.cu:111-205);
// this kernel multiplies nothing on the walk.  It tracks only the
// even-degree rows (odd rows never vanish), each by the offset
// u_r = t_r - deg_r / 2 (t_r = ones in plus columns) modulo 2^K, where
// 2^K > deg_r / 2 so that u_r = 0 exactly when s_r = 0.  The offsets are
// bit-sliced: plane b holds bit b of every tracked row's offset, one bit per
// row (one 32-bit word for up to 32 tracked rows, two for up to 64).  A Gray
// step adds or subtracts 1 in the tracked rows of the toggled column: a
// ripple through the K planes, two logic operations per plane and word.
// A state has a zero row exactly when some tracked row has all K plane bits
// clear: one OR chain per word.
//
// States with no zero row are appended to a per-warp queue in shared memory
// (a ballot gives each lane its slot).  Whenever 32 are queued, every lane
// of the warp evaluates one of them exactly: the row sums from the state's
// Gray word by popcount (s_r = deg_r - 2 popc(row_r & gray(g))), then the
// exact multi-word term of exact_glynn.cuh (row groups, signed running
// product, 64-bit column accumulators).  Walk and evaluation are both
// warp-uniform, so no lane idles while another evaluates.
//
// Rows are padded to NPAD (pad rows: degree 1, no toggled column, s = 1) so
// that one instantiation serves a range of orders; the walk itself runs the
// true order's 2^(n-1) states.  Accumulation, the block reduction and the
// per-block result slots are those of the exact kernel.
#pragma once

#include "exact_glynn.cuh"

namespace pg {

struct BinaryArgs {
    const uint64_t *rmask;     // [NPAD] toggled-column bits of each row (group order)
    const int32_t *deg;        // [NPAD] row degrees (pad rows 1)
    const uint64_t *cmask;     // [n-1] tracked rows of each toggled column (bit e)
    const uint64_t *trmask;    // [ntracked] toggled-column bits of each tracked row
    const int32_t *toff;       // [ntracked] deg_r - deg_r / 2 (offset of the all-plus state)
    int ntracked;              // even-degree rows, <= 32 W
    int n;
    unsigned long long *acc;   // [NL] per-word sums (exact kernel layout)
    int *status;
    unsigned long long *part;  // [NL][gridDim] per-block slots (exact_epilogue), or nullptr
    unsigned long long *next;  // chunk groups taken so far beyond each warp's first (the
                               // split instantiation): zero at launch, re-zeroed by the
                               // finishing kernel; unused without the split, where warp w
                               // walks groups w, w + warps, w + 2 warps, ...
    volatile const int *abort_flag;
    uint64_t chunks;
    int log_len;
    uint64_t chunk0;
    int threads;
};

constexpr int BIN_WARPS = 8;   // 256-thread blocks
constexpr int BIN_QCAP = 64;   // queue entries per warp (32 pending + one step's 32)

__host__ __device__ constexpr int binary_min_blocks(int NPAD) { return NPAD > 40 ? 1 : 2; }

template <int W, int K>
struct ZeroTracker {
    uint32_t p[K][W];
    uint32_t valid[W];        // tracked rows present in each word

    // t -= 1 (dec) or += 1 for the tracked rows in m, modulo 2^K
    __device__ __forceinline__ void step(uint64_t m, bool dec) {
        const uint32_t d = dec ? 0xffffffffu : 0u;
#pragma unroll
        for (int w = 0; w < W; w++) {
            uint32_t c = (uint32_t)(m >> (32 * w));
#pragma unroll
            for (int b = 0; b < K; b++) {
                const uint32_t t = (p[b][w] ^ d) & c;
                p[b][w] ^= c;
                c = t;
            }
        }
    }
    // true when no tracked row has offset 0 (no zero row sum)
    __device__ __forceinline__ bool nonzero() const {
        uint32_t zero = 0;
#pragma unroll
        for (int w = 0; w < W; w++) {
            uint32_t any = p[0][w];
#pragma unroll
            for (int b = 1; b < K; b++) any |= p[b][w];
            zero |= valid[w] & ~any;
        }
        return zero == 0;
    }
};

// Exact term of state g (or a zero term when !live) into the columns.  The
// Gray bits of g from the split up are those of the warp's current chunk
// group, and base[r] already holds deg_r minus twice the row's ones among
// them, so one 32-bit popcount per row remains.
template <int NPAD, int G>
__device__ __forceinline__ void binary_term(const uint64_t *rm, const int32_t *base, uint64_t g,
                                            bool live, uint32_t lowmask, uint64_t *col,
                                            int64_t &colt, bool first) {
    const uint32_t gl = (uint32_t)(g ^ (g >> 1)) & lowmask;
    int32_t s[NPAD];
#pragma unroll
    for (int r = 0; r < NPAD; r++) s[r] = base[r] - 2 * __popc((uint32_t)rm[r] & gl);
    if (!live) s[0] = 0;
    exact_term_col<NPAD, G, 0>(s, col, colt, (uint32_t)(g & 1), first);
}

// The same without the split (rare survivors, or windows whose first chunk
// is not a multiple of 32): the whole 64-bit Gray word is counted.
template <int NPAD, int G>
__device__ __forceinline__ void binary_term_full(const uint64_t *rm, const int32_t *deg, uint64_t g,
                                              bool live, uint64_t *col, int64_t &colt,
                                              bool first) {
    const uint64_t gm = g ^ (g >> 1);
    int32_t s[NPAD];
#pragma unroll
    for (int r = 0; r < NPAD; r++) s[r] = deg[r] - 2 * __popcll(rm[r] & gm);
    if (!live) s[0] = 0;
    exact_term_col<NPAD, G, 0>(s, col, colt, (uint32_t)(g & 1), first);
}

template <int NPAD, int G, int K, int W, bool SPLIT>
__global__ void __launch_bounds__(256, binary_min_blocks(NPAD))
binary_glynn_kernel(BinaryArgs a) {
    using S = ExactShape<NPAD, G>;
    constexpr int NL = S::NL, NR = S::NR, LOGU = 2, U = 1 << LOGU;
    constexpr int FOLD = 1 << EXACT_LOGU;   // terms the 64-bit columns hold between folds
    __shared__ uint64_t s_rm[NPAD];
    __shared__ int32_t s_deg[NPAD];
    __shared__ uint64_t s_cm[64];
    __shared__ uint64_t s_q[BIN_WARPS][BIN_QCAP];
    __shared__ int32_t s_base[BIN_WARPS][NPAD];
    exact_allow_dependents();
    for (int i = threadIdx.x; i < NPAD; i += blockDim.x) {
        s_rm[i] = a.rmask[i];
        s_deg[i] = a.deg[i];
    }
    for (int i = threadIdx.x; i < a.n - 1; i += blockDim.x) s_cm[i] = a.cmask[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t below = (1u << lane) - 1u;
    uint64_t *q = s_q[warp];

    uint32_t acc[NL];
#pragma unroll
    for (int l = 0; l < NL; l++) acc[l] = 0;
    uint64_t col[NR > 1 ? NR - 1 : 1];
    int64_t colt = 0;
    int terms = 0;       // terms in the columns since the last fold (warp-uniform)
    int qn = 0;          // queued states (warp-uniform)

    // Chunks are dealt in groups of 32 consecutive ones, lane l of a warp
    // taking the group's chunk l (so the step's column is warp-uniform and
    // every lane runs the same loop count, which the ballots need).  Each
    // warp walks its own group first and then, in the split instantiation
    // (survivors common), takes the next untaken group from a counter, one
    // atomic per 2^(log_len + 5) states.  The share of surviving states, and so the
    // exact evaluations, varies strongly along the walk with the signs of
    // the columns: a fixed deal (contiguous ranges, or round-robin with a
    // stride that is a multiple of 2^12 chunks, which pins twelve column
    // signs per warp) left some SMs with 40 % more instructions than the
    // mean.  When survivors are rare the walk dominates, the fixed
    // round-robin deal is balanced, and it saves the atomics (grid: 446 vs
    // 454 ms).  Each chunk starts from a closed-form tracker state.
    const uint64_t T = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t ngroups = (a.chunks + 31) >> 5;
    const uint64_t valid = a.ntracked >= 64 ? ~0ull : (1ull << a.ntracked) - 1;
    ZeroTracker<W, K> zt;
#pragma unroll
    for (int w = 0; w < W; w++) zt.valid[w] = (uint32_t)(valid >> (32 * w));
    // offsets at state `start`: u_e = toff_e - popc(row_e & gray(start)) mod 2^K
    auto init_tracker = [&](uint64_t start) {
        const uint64_t gs = start ^ (start >> 1);
        uint64_t planes[K];
#pragma unroll
        for (int b = 0; b < K; b++) planes[b] = 0;
        for (int e = 0; e < a.ntracked; e++) {
            const uint32_t u = (uint32_t)(a.toff[e] - __popcll(a.trmask[e] & gs));
#pragma unroll
            for (int b = 0; b < K; b++) planes[b] |= (uint64_t)((u >> b) & 1u) << e;
        }
#pragma unroll
        for (int w = 0; w < W; w++)
#pragma unroll
            for (int b = 0; b < K; b++) zt.p[b][w] = (uint32_t)(planes[b] >> (32 * w));
    };
    const uint32_t Q = (1u << a.log_len) >> LOGU;
    const uint64_t poll = a.log_len >= 16 ? 0 : (1ull << (16 - a.log_len)) - 1;
    const uint64_t cm0 = s_cm[0], cm1 = a.n - 1 > 1 ? s_cm[1] : 0;
    bool aborted = false;

    // The warp's lanes walk 32 consecutive chunks; when the window starts on
    // a multiple of 32 chunks, Gray bits from log_len + 5 up are common to
    // them, and the queue is emptied at the end of each chunk group so that
    // every queued state shares the group's high bits (s_base).  The host
    // turns this off when survivors are rare: the partial rounds of the
    // per-group flush then cost more than the popcounts they save.
    constexpr bool split = SPLIT;   // the host checks (chunk0 & 31) == 0, log_len + 5 <= 31
    const int sb = split ? a.log_len + 5 : 0;
    const uint32_t lowmask = split ? (1u << sb) - 1u : 0xffffffffu;
    const int32_t *base = split ? s_base[warp] : s_deg;

    auto evaluate = [&](bool flush) {
        __syncwarp();
        const bool live = lane < qn;
        if constexpr (SPLIT)
            binary_term<NPAD, G>(s_rm, base, live ? q[lane] : 0, live, lowmask, col, colt,
                                 terms == 0);
        else
            binary_term_full<NPAD, G>(s_rm, s_deg, live ? q[lane] : 0, live, col, colt,
                                      terms == 0);
        if (++terms == FOLD) {
            FoldCols<NR, NL>::apply(acc, col, colt);
            terms = 0;
        }
        __syncwarp();
        if (!flush) {
            if (lane + 32 < qn) q[lane] = q[lane + 32];
            qn -= 32;
        }
        __syncwarp();
    };

    // split: group grp (the warp's own first, then from the counter);
    // otherwise round k of the round-robin deal (chunk k T + tid)
    const uint64_t kmax = (a.chunks + T - 1) / T;
    uint64_t grp = tid >> 5;
    for (uint64_t k = 0; SPLIT ? grp < ngroups : k < kmax; k++) {
        if (k != 0 && (k & poll) == 0 && __any_sync(0xffffffffu, *a.abort_flag != 0)) {
            aborted = true;
            break;
        }
        // the next group is taken now and used after this one, so the
        // atomic's round trip overlaps the walk
        unsigned long long nx = 0;
        if constexpr (SPLIT) {
            if (lane == 0) nx = (T >> 5) + atomicAdd(a.next, 1ull);
        }
        const uint64_t ci = SPLIT ? (grp << 5) + lane : k * T + tid;
        const bool act = ci < a.chunks;
        const uint64_t c = a.chunk0 + ci;
        if (act) init_tracker(c << a.log_len);
        if (split) {
            // the group's common Gray bits (the queue is empty here)
            const uint64_t g0 = c << a.log_len;
            const uint64_t gh = (g0 ^ (g0 >> 1)) & ~(uint64_t)lowmask;
            for (int r = lane; r < NPAD; r += 32) s_base[warp][r] = s_deg[r] - 2 * __popcll(s_rm[r] & gh);
            __syncwarp();
        }
        const uint32_t hib = (uint32_t)(c & 1) << a.log_len;
        for (uint32_t qq = 0; qq < Q; qq++) {
            const uint32_t g32 = (qq << LOGU) | hib;
#pragma unroll
            for (int r = 0; r < U; r++) {
                // the chunk's first state is the initialised one
                const bool step = act && (r != 0 || qq != 0);
                uint64_t m = 0;
                bool dec = false;
                if (r != 0) {
                    const int j = exact_ctz_small(r);
                    m = j == 0 ? cm0 : cm1;
                    dec = (j + 1 < LOGU) ? ((r >> (j + 1)) & 1) == 0 : ((g32 >> LOGU) & 1) == 0;
                } else if (qq != 0) {
                    const int j = __ffs(qq) - 1 + LOGU;
                    m = s_cm[j];
                    dec = ((g32 >> (j + 1)) & 1) == 0;
                }
                if (step) zt.step(m, dec);
                const bool nz = act && zt.nonzero();
                const uint32_t mask = __ballot_sync(0xffffffffu, nz);
                if (mask) {
                    if (nz) q[qn + __popc(mask & below)] = ((c << a.log_len) | g32 | (uint32_t)r);
                    qn += __popc(mask);
                    if (qn >= 32) evaluate(false);
                }
            }
        }
        if (split && qn > 0) {      // the next group has other high bits
            evaluate(true);
            qn = 0;
        }
        if constexpr (SPLIT) grp = __shfl_sync(0xffffffffu, nx, 0);
    }
    if (qn > 0) evaluate(true);
    if (terms > 0) FoldCols<NR, NL>::apply(acc, col, colt);

    // block reduction and result words: as the exact kernel
    __shared__ long long red[8][NL];
    __shared__ int any_abort;
    if (threadIdx.x == 0) any_abort = 0;
    __syncthreads();
    if (aborted) any_abort = 1;
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

template <int NPAD, int G, int K, int W>
cudaError_t launch_binary_glynn(const BinaryArgs &args, bool split, int blocks,
                                cudaStream_t stream) {
    if (split)
        binary_glynn_kernel<NPAD, G, K, W, true><<<blocks, args.threads, 0, stream>>>(args);
    else
        binary_glynn_kernel<NPAD, G, K, W, false><<<blocks, args.threads, 0, stream>>>(args);
    return cudaGetLastError();
}

template <int NPAD, int G, int K, int W>
int occupancy_binary_glynn() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, binary_glynn_kernel<NPAD, G, K, W, true>, 256, 0) != cudaSuccess)
        return 1;
    return nb < 1 ? 1 : nb;
}

// Compiled shapes (binary_inst_*.cu): NPAD in {32, 40, 48}, G in {5, 6, 7,
// 8, 10}, K in {2, 3, 4, 5} offset planes, W = 1 tracking word (2 for
// NPAD 40 and 48 with more than 32 even-degree rows).  Orders below
// BINARY_MIN_N, and matrices whose sampled share of states without a zero
// row exceeds BINARY_MAX_SURVIVORS, use the exact kernel.  EXACT_BINARY=0
// sends every 0/1 matrix to the exact kernel (for comparisons).
constexpr int BINARY_MIN_N = 24;
constexpr double BINARY_MAX_SURVIVORS = 0.25;
#ifndef EXACT_BINARY
#define EXACT_BINARY 1
#endif
int binary_npad(int n);
bool binary_compiled(int NPAD, int G, int K, int W);
cudaError_t launch_binary_any(int NPAD, int G, int K, int W, const BinaryArgs &args, bool split,
                              int blocks, cudaStream_t stream);
int occupancy_binary_any(int NPAD, int G, int K, int W);

}  // namespace pg
