// pg_exact_permanent_noalloc: the exact Glynn engine for callers that cannot
// allocate memory.
//
// Some callers cannot call cudaMalloc: plug-ins whose host process owns
// every device allocation through its own pool (a cudaMalloc behind the
// pool's back breaks its accounting or fails outright), and services that
// reserve a fixed device-memory budget at start-up and must not grow it
// afterwards.  This entry point runs the same kernel as pg_exact_permanent
// (integer rows only, so at orders 24..32 it is somewhat slower than the
// allocating path, which can keep three rows of each group of four in FP32),
// but its scratch (column tables, initial row sums, the per-word
// accumulators and the status word) lives in one file-scope __device__
// array of fixed size, so the call allocates nothing: no cudaMalloc or
// cudaFree, no pinned or host heap buffers, no streams.
//
// Limits and sharing rules:
//   * the scratch holds at most PG_NOALLOC_SCRATCH_BYTES (32 KiB); every
//     order the exact engine takes (2..48) fits, and the byte count of each
//     request is still checked against the array before any device work;
//   * every loaded copy of the library keeps this array on every GPU that
//     loads it, until the process exits;
//   * all calls share the array and each call leaves its contents behind;
//     the call zeroes the accumulator and status words itself, but two
//     calls whose work overlaps on the GPU (different streams or host
//     threads) race on the same words and corrupt each other's result —
//     serialise them;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, that device current) and keeps
//     it for the life of the process.  Calls after cudaDeviceReset on that
//     device are not supported (the cached address belongs to the old
//     context);
//   * the call copies the inputs from and the result to host memory and
//     synchronises `stream` before it returns;
//   * pg_abort() reaches this entry point only when the process-wide abort
//     word already exists (created by pg_abort, pg_clear_abort or any
//     allocating entry point); this entry point never creates it, and
//     without it the launch runs to completion.
#include "pg_internal.h"
#include "exact_glynn.cuh"

#include <cmath>
#include <cstring>
#include <mutex>

#define PG_NOALLOC_SCRATCH_BYTES (32 * 1024)
#define PG_NOALLOC_MAX_DEVICES 64

namespace pg {

// Scratch: [tables | init | acc words | status | zero word (abort flag when
// the process has no abort word yet) | result words, status]
static __device__ __align__(256) unsigned char g_noalloc_scratch[PG_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[PG_NOALLOC_MAX_DEVICES] = {nullptr};

static int noalloc_scratch(unsigned char **out) {
    int dev = 0;
    PG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= PG_NOALLOC_MAX_DEVICES)
        return fail(PG_ERANGE, "device ordinal beyond the no-alloc table");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_noalloc_ptr[dev] = p;
    }
    *out = (unsigned char *)g_noalloc_ptr[dev];
    return PG_OK;
}

static size_t na_align(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace pg

extern "C" int pg_exact_permanent_noalloc(const int64_t *A, int n, uint32_t *out,
                                          int limbs, void *stream) {
    using namespace pg;
    if (n < 2 || n > 48) return fail(PG_ERANGE, "no-alloc exact engine supports 2 <= n <= 48");
    if (!A || !out || limbs < 1) return fail(PG_EINVAL, "null argument");

    // row bounds and grouping, on the stack
    uint64_t B[48];
    double bits = 0;
    for (int i = 0; i < n; i++) {
        unsigned __int128 s = 0;
        for (int j = 0; j < n; j++) {
            const int64_t v = A[(size_t)i * n + j];
            s += v < 0 ? (unsigned __int128)(-(__int128)v) : (unsigned __int128)v;
        }
        if (s >= ((unsigned __int128)1 << 30))
            return fail(PG_EOVERFLOW, "row-sum bound exceeds the exact engine's fixed widths");
        B[i] = (uint64_t)s;
        bits += std::log2(B[i] ? (double)B[i] : 1.0);
    }
    if (32.0 * limbs < bits + 2)
        return fail(PG_ERANGE, "output limb count too small for the permanent bound");
    int order[48], G = 0;
    for (int g = EXACT_MAX_G; g >= 1 && !G; g--) {
        if (!exact_compiled(n, g)) continue;
        if (!exact_group_rows(B, n, g, order)) continue;
        G = g;
    }
    if (!G) return fail(PG_EOVERFLOW, "row-sum bound exceeds the exact engine's fixed widths");

    const int NCOL = n - 1, NP = (n + 3) & ~3;
    const int NG = (n + G - 1) / G, NL = NG + (n > 32 ? 2 : 1);
    const size_t off_init = na_align((size_t)NCOL * 2 * NP * 4);
    const size_t off_acc = na_align(off_init + (size_t)NP * 4);
    const size_t off_status = na_align(off_acc + (size_t)NL * 8);
    const size_t off_zero = off_status + 8;
    const size_t off_out = na_align(off_zero + 8);
    const size_t total = na_align(off_out + (size_t)(NL + 1) * 8);
    if (total > PG_NOALLOC_SCRATCH_BYTES)
        return fail(PG_ERANGE, "problem exceeds the no-alloc scratch (32 KiB)");

    unsigned char *scratch = nullptr;
    int st = noalloc_scratch(&scratch);
    if (st != PG_OK) return st;
    DeviceInfo dev;
    st = device_info(&dev);
    if (st != PG_OK) return st;

    // host image of [tables | init] on the stack, then one pageable copy
    static_assert(PG_NOALLOC_SCRATCH_BYTES % 4 == 0, "scratch is whole words");
    int32_t image[PG_NOALLOC_SCRATCH_BYTES / 4];
    std::memset(image, 0, off_acc);
    int32_t *tab = image;
    int32_t *init = image + off_init / 4;
    for (int ii = 0; ii < n; ii++) {
        const int64_t *row = A + (size_t)order[ii] * n;
        int64_t sum = 0;
        for (int j = 0; j < n; j++) sum += row[j];
        init[ii] = (int32_t)sum;
        for (int j = 0; j < NCOL; j++) {
            tab[(2 * j + 0) * NP + ii] = (int32_t)(2 * row[j]);
            tab[(2 * j + 1) * NP + ii] = (int32_t)(-2 * row[j]);
        }
    }
    cudaStream_t s = (cudaStream_t)stream;
    PG_CUDA(cudaMemcpyAsync(scratch, image, off_acc, cudaMemcpyHostToDevice, s));
    // accumulators, status, result words and the always-zero abort word
    // start at zero
    PG_CUDA(cudaMemsetAsync(scratch + off_acc, 0, total - off_acc, s));

    // launch shape as in the allocating path
    const int occ = occupancy_exact_any(n, G);
    const int log_states = n - 1;
    uint64_t blocks = 0;
    int threads = 256, log_len = 0;
    exact_launch_shape(log_states, occ, dev.sm_count, &blocks, &threads, &log_len);

    ExactArgs args;
    args.tab = (const int32_t *)scratch;
    args.init = (const int32_t *)(scratch + off_init);
    args.acc = (unsigned long long *)(scratch + off_acc);
    args.status = (int *)(scratch + off_status);
    volatile int *abort_word = abort_flag_device_if_created();
    args.abort_flag = abort_word ? (volatile const int *)abort_word
                                 : (volatile const int *)(scratch + off_zero);
    args.chunks = 1ull << (log_states - log_len);
    args.log_len = log_len;
    args.chunk0 = 0;
    args.threads = threads;
    PG_CUDA(launch_exact_any(n, G, args, (int)blocks, s));
    PG_CUDA(exact_finish(nullptr, (int)blocks, NL, args.acc, args.status,
                         (unsigned long long *)(scratch + off_out), s));

    long long acc[64];          // NL + 1 <= 19 for every compiled shape: words, status
    PG_CUDA(cudaMemcpyAsync(acc, scratch + off_out, (size_t)(NL + 1) * 8, cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    if (acc[NL]) return fail(PG_EABORT, "no-alloc exact launch aborted by pg_abort()");

    // carry the per-word sums into S (two's complement) and shift by n-1
    uint32_t S[72] = {0};
    const int W = NL + 3;
    for (int l = 0; l < NL; l++) {
        const long long v = acc[l];
        const uint32_t ext = v < 0 ? 0xffffffffu : 0u;
        uint64_t carry = 0;
        for (int i = l; i < W; i++) {
            const uint32_t add = i == l ? (uint32_t)(uint64_t)v
                               : i == l + 1 ? (uint32_t)((uint64_t)v >> 32) : ext;
            const uint64_t t = (uint64_t)S[i] + add + carry;
            S[i] = (uint32_t)t;
            carry = t >> 32;
        }
    }
    const int sh = n - 1;
    for (int b = 0; b < sh; b++)
        if ((S[b >> 5] >> (b & 31)) & 1)
            return fail(PG_EINTERNAL, "Glynn sum not divisible by 2^(n-1)");
    const uint32_t ext = (S[W - 1] >> 31) ? 0xffffffffu : 0u;
    for (int i = 0; i < limbs; i++) {
        const int bit = 32 * i + sh;
        const int wi = bit >> 5, bo = bit & 31;
        const uint32_t lo = wi < W ? S[wi] : ext;
        const uint32_t hi = wi + 1 < W ? S[wi + 1] : ext;
        out[i] = bo ? (lo >> bo) | (hi << (32 - bo)) : lo;
    }
    return PG_OK;
}
