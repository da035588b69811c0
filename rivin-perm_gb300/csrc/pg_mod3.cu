// Permanent modulo 3 by Ryser's formula with bit-sliced F_3 row sums.
//
//   per(A) = (-1)^n sum_{S subset of columns} (-1)^|S| prod_i sum_{j in S} a_ij
// over F_3 (rivin-perm perm_mod3.py:143-228, perm_mod3_omp.c, CUDA kernel
// perm_mod3_cuda.cu:52-131).  Each element of F_3 is two bits (magnitude,
// sign): 0 = (0, either), 1 = (1,0), -1 = 2 = (1,1); the n row sums of a
// subset are two n-bit words, and adding or subtracting a canonical column
// is a few bitwise operations on them (the bipedal formulas of
// arXiv:2407.20205; their truth table over every row-sum encoding and
// canonical column is checked on the host in the tests).  A subset
// contributes iff every row sum is nonzero (magnitude word full), and then
// every sign bit is meaningful: sign (-1)^(popcount(sign word) + |S|).
//
// GB300 organisation: the 2^n Gray-ordered subsets are cut into aligned
// chunks, each thread walks a contiguous balanced range of chunks; inside a
// chunk the walk is unrolled by 8, so the toggled column of 7 of every 8
// steps (columns 0..2) is a compile-time register operand and only the
// eighth reads shared memory (uniform across the warp).  Words are 32-bit
// for n <= 32 (one ALU op per bitwise step) and 64-bit above.  Each thread
// counts its terms as 1 (for +1) or 2 (for -1), the count mod 3 is reduced
// per block and added atomically.
#include "pg_internal.h"

#include <cstring>

namespace pg {

struct Mod3Args {
    const uint64_t *cols;     // [2][n]: magnitude words, then sign words
    int n;
    uint64_t chunks;
    int log_len;              // >= 3
    unsigned long long *acc;  // zeroed
    int *status;
    volatile const int *abort_flag;
};

// row sums (m, s) += or -= column (cm, cs) over F_3, bitwise per row
template <typename W>
__device__ __forceinline__ void f3_add(W &m, W &s, W cm, W cs) {
    const W t = m ^ s ^ cs;
    const W mo = (cm & t) | (m ^ cm);
    s = (cm & t) ^ s;
    m = mo;
}
template <typename W>
__device__ __forceinline__ void f3_sub(W &m, W &s, W cm, W cs) {
    const W t = s ^ cs;
    const W mo = (m & t) | (m ^ cm);
    s = (m & t) ^ (cm ^ cs);
    m = mo;
}

template <typename W>
__device__ __forceinline__ int f3_parity(W s) {
    if constexpr (sizeof(W) == 8) return __popcll((unsigned long long)s) & 1;
    else return __popc((unsigned)s) & 1;
}

template <typename W>
__global__ void __launch_bounds__(256) mod3_kernel(Mod3Args a) {
    constexpr int LOGU = 3, U = 1 << LOGU;
    __shared__ W cm_s[64], cs_s[64];
    const int n = a.n;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        cm_s[j] = (W)a.cols[j];
        cs_s[j] = (W)a.cols[n + j];
    }
    __syncthreads();
    const W mask = (W)(n >= 64 ? ~0ull : ((1ull << n) - 1));
    W c0m = cm_s[0], c0s = cs_s[0], c1m = cm_s[1], c1s = cs_s[1], c2m = cm_s[2], c2s = cs_s[2];

    const uint64_t T = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t c_begin = tid * a.chunks / T;
    const uint64_t c_end = (tid + 1) * a.chunks / T;
    unsigned long long count = 0;   // sum of 1 (term +1) or 2 (term -1)
    bool aborted = false;
    if (c_begin < c_end) {
        W m = 0, s = 0;
        const uint64_t start = c_begin << a.log_len;
        const uint64_t gs = start ^ (start >> 1);
        for (int j = 0; j < n; j++)
            if ((gs >> j) & 1) f3_add(m, s, cm_s[j], cs_s[j]);
        const uint32_t blocks = (1u << a.log_len) >> LOGU;
        // the host-mapped abort word is read once per 2^20 subsets (per chunk
        // for longer chunks), from the thread's second period on
        const uint64_t poll = a.log_len >= 20 ? 0 : (1ull << (20 - a.log_len)) - 1;
        for (uint64_t c = c_begin; c < c_end; c++) {
            if (c != c_begin && ((c - c_begin) & poll) == 0 && *a.abort_flag) {
                aborted = true;
                break;
            }
            for (uint32_t q = 0; q < blocks; q++) {
                const uint64_t base = (c << a.log_len) | ((uint64_t)q << LOGU);
#pragma unroll
                for (int r = 0; r < U; r++) {
                    const uint64_t i = base | (uint64_t)r;
                    if (r == 0) {
                        if (i != start) {
                            const int j = __ffsll((long long)i) - 1;   // >= LOGU
                            if (((i >> (j + 1)) & 1) == 0) f3_add(m, s, cm_s[j], cs_s[j]);
                            else f3_sub(m, s, cm_s[j], cs_s[j]);
                        }
                    } else {
                        const int j = r & 1 ? 0 : (r & 2 ? 1 : 2);
                        // added when bit j+1 of i is 0 (bit LOGU of i for j = 2)
                        const bool add = j + 1 < LOGU ? ((r >> (j + 1)) & 1) == 0
                                                      : ((i >> LOGU) & 1) == 0;
                        const W cmj = j == 0 ? c0m : (j == 1 ? c1m : c2m);
                        const W csj = j == 0 ? c0s : (j == 1 ? c1s : c2s);
                        if (add) f3_add(m, s, cmj, csj);
                        else f3_sub(m, s, cmj, csj);
                    }
                    // Bits above row n stay 0 in both words, so "every row sum
                    // nonzero" is m == mask.  That is rare (about (2/3)^n for
                    // random entries), so the sign work sits behind a branch
                    // that is almost never taken.
                    // Subset sign (-1)^|S| = (-1)^popcount(gray(i)) = (-1)^r.
                    if (m == mask) count += (unsigned long long)(1 + (f3_parity(s) ^ (r & 1)));
                }
            }
        }
    }
    count %= 3;
    __shared__ unsigned long long red[8];
    __shared__ int any_abort;
    if (threadIdx.x == 0) any_abort = 0;
    __syncthreads();
    if (aborted) any_abort = 1;
    for (int off = 16; off > 0; off >>= 1) count += __shfl_down_sync(0xffffffffu, count, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = count;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        atomicAdd(a.acc, t);
        if (any_abort) atomicExch(a.status, 1);
    }
}

template <typename W>
static cudaError_t launch_mod3(const Mod3Args &a, int sm_count, cudaStream_t s) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mod3_kernel<W>, 256, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    uint64_t blocks = (uint64_t)per_sm * sm_count;
    const uint64_t max_blocks = (a.chunks + 255) / 256;
    if (blocks > max_blocks) blocks = max_blocks;
    if (blocks < 1) blocks = 1;
    mod3_kernel<W><<<(unsigned)blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

// perm(A) mod 3 from the F_3 column encodings (n >= 3).
static int mod3_impl(const uint64_t *mags, const uint64_t *sgns, int n, int *out) {
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    const size_t off_acc = 2 * 64 * 8, off_status = off_acc + 64, total = off_status + 64;
    Workspace *ws;
    st = workspace(&ws, total, total);
    if (st != PG_OK) return st;
    char *h = (char *)ws->host;
    char *d = (char *)ws->dev;
    std::memset(h, 0, total);
    std::memcpy(h, mags, (size_t)n * 8);
    std::memcpy(h + (size_t)n * 8, sgns, (size_t)n * 8);
    // 2^n subsets in at most 2^24 aligned chunks of >= 8 subsets
    const ChunkPlan pl = plan_chunks(n, 3, 1ull << 22);
    Mod3Args a;
    a.cols = (const uint64_t *)d;
    a.n = n;
    a.chunks = pl.chunks;
    a.log_len = pl.log_len;
    a.acc = (unsigned long long *)(d + off_acc);
    a.status = (int *)(d + off_status);
    a.abort_flag = abort_dev;
    PG_CUDA(cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, ws->stream));
    if (n <= 32) PG_CUDA((launch_mod3<uint32_t>(a, dev.sm_count, ws->stream)));
    else PG_CUDA((launch_mod3<uint64_t>(a, dev.sm_count, ws->stream)));
    PG_CUDA(cudaMemcpyAsync(h + off_acc, d + off_acc, total - off_acc, cudaMemcpyDeviceToHost,
                            ws->stream));
    PG_CUDA(cudaStreamSynchronize(ws->stream));
    if (*(int *)(h + off_status)) return fail(PG_EABORT, "launch aborted by pg_abort()");
    const unsigned long long total3 = *(unsigned long long *)(h + off_acc) % 3;
    *out = (int)((n & 1) ? (3 - total3) % 3 : total3);
    return PG_OK;
}

}  // namespace pg

extern "C" int pg_permanent_mod3_cols(const uint64_t *col_mags, const uint64_t *col_sgns,
                                      int n, int *out) {
    using namespace pg;
    if (!out) return fail(PG_EINVAL, "null argument");
    if (n < 0 || n >= 64) return fail(PG_ERANGE, "n must satisfy 0 <= n < 64");
    if (n == 0) { *out = 1; return PG_OK; }
    if (!col_mags || !col_sgns) return fail(PG_EINVAL, "column encodings must not be NULL");
    const uint64_t mask = (1ull << n) - 1;
    for (int j = 0; j < n; j++)
        if ((col_mags[j] & ~mask) || (col_sgns[j] & ~col_mags[j]))
            return fail(PG_EINVAL, "column encodings out of range (sign bit without magnitude "
                                   "or row >= n)");
    if (n <= 2) {
        // per = a00 (n = 1) or a00 a11 + a01 a10 (n = 2), elements of F_3
        auto el = [&](int i, int j) -> int {
            if (!((col_mags[j] >> i) & 1)) return 0;
            return ((col_sgns[j] >> i) & 1) ? 2 : 1;
        };
        *out = n == 1 ? el(0, 0) : (el(0, 0) * el(1, 1) + el(0, 1) * el(1, 0)) % 3;
        return PG_OK;
    }
    return mod3_impl(col_mags, col_sgns, n, out);
}

extern "C" int pg_permanent_mod3(const int64_t *A, int n, int *out) {
    using namespace pg;
    if (!out) return fail(PG_EINVAL, "null argument");
    if (n < 0 || n >= 64) return fail(PG_ERANGE, "n must satisfy 0 <= n < 64");
    if (n == 0) { *out = 1; return PG_OK; }
    if (!A) return fail(PG_EINVAL, "matrix must not be NULL");
    uint64_t mags[64] = {0}, sgns[64] = {0};
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            const int64_t r = A[(size_t)i * n + j] % 3;
            const int v = (int)(r < 0 ? r + 3 : r);
            if (v) mags[j] |= 1ull << i;
            if (v == 2) sgns[j] |= 1ull << i;
        }
    return pg_permanent_mod3_cols(mags, sgns, n, out);
}
