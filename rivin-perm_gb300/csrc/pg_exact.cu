// Host side of the exact Glynn engine: bound check, row grouping, tables,
// launch, and the carry of per-word sums into per(A) = S / 2^(n-1).
#include "pg_internal.h"
#include "exact_glynn.cuh"
#include "binary_glynn.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace pg {

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Greedy grouping: rows in descending bound order, each into the open group
// with the smallest log-product.  With small_last the last group is first
// filled with the rows of smallest bound (it multiplies into the columns).
static bool try_grouping(const uint64_t *B, int n, int G, bool small_last, int *order) {
    const int NG = (n + G - 1) / G;
    const int last_cap = n - (NG - 1) * G;
    int idx[48], cnt[48] = {0}, mem[48][EXACT_MAX_G];
    double lp[48] = {0};
    for (int i = 0; i < n; i++) idx[i] = i;
    for (int i = 1; i < n; i++)                    // stable, descending B
        for (int k = i; k > 0 && B[idx[k]] > B[idx[k - 1]]; k--) std::swap(idx[k], idx[k - 1]);
    int rows = n;
    if (small_last && NG > 1) {
        for (int t = 0; t < last_cap; t++) mem[NG - 1][cnt[NG - 1]++] = idx[n - 1 - t];
        rows = n - last_cap;
    }
    for (int i = 0; i < rows; i++) {
        int best = -1;
        for (int g = 0; g < NG; g++) {
            if (cnt[g] >= (g == NG - 1 ? last_cap : G)) continue;
            if (best < 0 || lp[g] < lp[best]) best = g;
        }
        mem[best][cnt[best]++] = idx[i];
        lp[best] += std::log2((double)(B[idx[i]] ? B[idx[i]] : 1));
    }
    for (int g = 0; g < NG; g++) {
        unsigned __int128 prod = 1;
        for (int t = 0; t < cnt[g]; t++) {
            prod *= (B[mem[g][t]] ? B[mem[g][t]] : 1);
            if (prod >= ((unsigned __int128)1 << 31)) return false;
        }
        if (g == NG - 1 && prod > EXACT_LAST_GROUP_MAX) return false;
    }
    int w = 0;
    for (int g = 0; g < NG; g++)
        for (int t = 0; t < cnt[g]; t++) order[w++] = mem[g][t];
    return true;
}

bool exact_group_rows(const uint64_t *B, int n, int G, int *order) {
    if (n < 1 || n > 48 || G < 1 || G > EXACT_MAX_G) return false;
    return try_grouping(B, n, G, false, order) || try_grouping(B, n, G, true, order);
}

// Picks the largest compiled group size that admits a grouping (fewest
// product words).
static int choose_group(const int64_t *A, int n, std::vector<int> *order) {
    if (n < 2 || n > 48) return 0;
    std::vector<uint64_t> B(n);
    for (int i = 0; i < n; i++) {
        unsigned __int128 s = 0;
        for (int j = 0; j < n; j++) {
            const int64_t v = A[(size_t)i * n + j];
            s += v < 0 ? (unsigned __int128)(-(__int128)v) : (unsigned __int128)v;
        }
        if (s >= ((unsigned __int128)1 << 30)) return 0;
        B[i] = (uint64_t)s;
    }
    order->resize(n);
    for (int G = EXACT_MAX_G; G >= 1; G--) {
        if (!exact_compiled(n, G)) continue;
        if (exact_group_rows(B.data(), n, G, order->data())) return G;
    }
    return 0;
}

// bits of prod_i max(1, B_i), i.e. of the Hadamard-type bound of perm.py:939-953
static int bound_bits(const int64_t *A, int n) {
    double bits = 0;
    for (int i = 0; i < n; i++) {
        double s = 0;
        for (int j = 0; j < n; j++) s += std::fabs((double)A[(size_t)i * n + j]);
        bits += std::log2(s < 1 ? 1 : s);
    }
    return (int)std::ceil(bits + 1e-9);
}

// words += v * 2^(32*pos) in W-word two's complement
static void add_i64_at(std::vector<uint32_t> &w, int pos, long long v) {
    const int W = (int)w.size();
    const uint32_t ext = v < 0 ? 0xffffffffu : 0u;
    uint64_t carry = 0;
    for (int i = pos; i < W; i++) {
        uint32_t add = i == pos ? (uint32_t)(uint64_t)v
                     : i == pos + 1 ? (uint32_t)((uint64_t)v >> 32) : ext;
        const uint64_t t = (uint64_t)w[i] + add + carry;
        w[i] = (uint32_t)t;
        carry = t >> 32;
    }
}


void exact_launch_shape(int log_states, int occ, int sm_count, uint64_t *blocks,
                        int *threads, int *log_len) {
    const uint64_t states = 1ull << log_states;
    const uint64_t sms = (uint64_t)(sm_count < 1 ? 1 : sm_count);
    const uint64_t cap = (uint64_t)(occ < 1 ? 1 : occ) * sms * 256;
    uint64_t T = states / EXACT_MIN_THREAD_STATES;
    if (T > cap) T = cap;
    uint64_t B;
    int tpb;
    if (T / sms < 32) {                       // fewer warps than SMs
        tpb = 32;
        B = T / 32 ? T / 32 : 1;
    } else {                                  // the same whole warps on every SM
        const uint64_t per_sm = (T / sms) & ~31ull;
        const uint64_t k = (per_sm + 255) / 256;
        tpb = (int)((per_sm / k) & ~31ull);
        B = sms * k;
    }
    const uint64_t TT = B * (uint64_t)tpb;
    int log_T = 0;
    while ((2ull << log_T) <= TT) log_T++;
    // ~128 chunks per thread on long walks; shorter walks keep chunks of 64
    // states while every thread still gets >= 6 of them, and below that go
    // down to 2^EXACT_MIN_CHUNK_LOG states so the per-thread ranges stay
    // even (the chunk's first step is the only divergent one)
    int ll = log_states - (log_T + 7);
    int fit = 0;
    while (fit < 6 && (states >> (fit + 1)) / TT >= 6) fit++;
    const int want = EXACT_MIN_CHUNK_LOG > EXACT_LOGU ? EXACT_MIN_CHUNK_LOG : EXACT_LOGU;
    const int floor_len = fit > want ? fit : want;
    const int min_len = log_states < floor_len ? log_states : floor_len;
    if (ll < min_len) ll = min_len;
    if (ll > 30) ll = 30;
    if (ll < 1) ll = 1;
    *blocks = B;
    *threads = tpb;
    *log_len = ll;
}

// Everything one exact evaluation needs, built once on the host.
// Float rows for group size G: within each group the rows are ordered by
// increasing bound, and the first exact_float_rows(n, G, FR, g) of them must
// have bounds below 2^24 (exact FP32 sums) with a product below 2^22 (exact
// FP32 product, converted by the 1.5 * 2^23 add).  Reorders `order` in
// place (group membership is unchanged) and returns true when every group
// qualifies.
bool exact_frows_arrange(const int64_t *A, int n, int G, int FR, int *order_io) {
    std::vector<int> ord(order_io, order_io + n);
    std::vector<int> *order = &ord;
    if (FR <= 0) return false;
    std::vector<uint64_t> B(n);
    for (int i = 0; i < n; i++) {
        uint64_t s = 0;
        for (int j = 0; j < n; j++) {
            const int64_t v = A[(size_t)i * n + j];
            s += (uint64_t)(v < 0 ? -v : v);
        }
        B[i] = s;
    }
    std::vector<int> o = *order;
    const int NG = (n + G - 1) / G;
    for (int g = 0; g < NG; g++) {
        const int sz = exact_group_size(n, G, g), nf = exact_float_rows(n, G, FR, g);
        int *grp = o.data() + g * G;
        std::sort(grp, grp + sz, [&](int x, int y) { return B[x] < B[y]; });
        unsigned __int128 prod = 1;
        for (int t = 0; t < nf; t++) {
            if (B[grp[t]] >= (1ull << 24)) return false;
            prod *= (B[grp[t]] ? B[grp[t]] : 1);
        }
        if (prod >= ((unsigned __int128)1 << 22)) return false;
    }
    std::copy(o.begin(), o.end(), order_io);
    return true;
}

static uint32_t float_bits(int64_t v) {
    const float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

struct ExactPlan {
    int n = 0, G = 0, NG = 0, NL = 0, need_bits = 0;
    int fr = 0;                  // float rows per group (0: integer rows)
    // bit-sliced 0/1 kernel (binary_glynn.cuh): offset planes K > 0,
    // tracking words W, tracked (even-degree) rows, padded rows
    int planes = 0, words_tracked = 0, ntracked = 0, npad = 0, bin_split = 0;
    size_t off_deg = 0, off_cm = 0, off_trm = 0, off_toff = 0;
    ChunkPlan chunks{};
    uint64_t chunk0 = 0;
    uint64_t blocks = 0;
    int threads = 256;
    size_t off_acc = 0, off_status = 0, off_out = 0, off_part = 0, total = 0;
    std::vector<char> image;     // host image of [tab | init | acc | status]
    // device side (owned by a plan object, or borrowed from a workspace)
    char *dev = nullptr;
    char *host = nullptr;        // pinned staging, >= total bytes
    bool owns = false;
    cudaStream_t stream = nullptr;
    volatile int *abort_dev = nullptr;
};

// The bit-sliced kernel for a 0/1 matrix of order BINARY_MIN_N..48: the
// even-degree rows are tracked for zero row sums, rows are padded to NPAD
// (degree 1, no columns) and grouped by degree like the exact kernel; the
// last column keeps the fixed sign.  The share of states with no zero row
// is estimated from 1024 sampled states: above BINARY_MAX_SURVIVORS the
// exact evaluations would cost more than the general kernel, which then
// runs (as it does when the matrix is not 0/1 or no compiled shape fits).
static bool plan_build_binary(const int64_t *A, int n, ExactPlan *P) {
    if (!EXACT_BINARY || n < BINARY_MIN_N || n > 48) return false;
    for (size_t i = 0; i < (size_t)n * n; i++)
        if (A[i] != 0 && A[i] != 1) return false;
    const int NPAD = binary_npad(n);
    std::vector<uint64_t> deg(NPAD, 1), rows(NPAD, 0);
    std::vector<int> tracked;
    int maxh = 0;
    for (int i = 0; i < n; i++) {
        uint64_t d = 0, m = 0;
        for (int j = 0; j < n; j++) {
            d += (uint64_t)A[(size_t)i * n + j];
            if (j < n - 1 && A[(size_t)i * n + j]) m |= 1ull << j;
        }
        deg[i] = d;
        rows[i] = m;
        if (d % 2 == 0) {
            tracked.push_back(i);
            maxh = std::max(maxh, (int)(d / 2));
        }
    }
    if (tracked.empty()) return false;          // no row can vanish: every state counts
    int K = 2;
    while ((1 << K) <= maxh) K++;
    const int W = tracked.size() > 32 ? 2 : 1;
    // sampled share of states with no zero row (fixed LCG, Gray words)
    uint64_t x = 0x9e3779b97f4a7c15ull;
    int survive = 0;
    const int samples = 1024;
    const uint64_t state_mask = (1ull << (n - 1)) - 1;
    for (int t = 0; t < samples; t++) {
        x = x * 6364136223846793005ull + 1442695040888963407ull;
        const uint64_t g = (x >> 11) & state_mask, gm = g ^ (g >> 1);
        bool zero = false;
        for (int r : tracked)
            if (2 * (uint64_t)__builtin_popcountll(rows[r] & gm) == deg[r]) { zero = true; break; }
        survive += !zero;
    }
    if (survive > BINARY_MAX_SURVIVORS * samples) return false;
    // evaluation from the warp's common high bits pays from a survivor
    // share of about 1/64 (40x40 Bernoulli(1/2): ~8 %; the grid: ~0.1 %)
    P->bin_split = survive * 64 >= samples;
    std::vector<int> order(NPAD);
    int G = 0;
    for (int g : {10, 8, 7, 6, 5}) {
        if (!binary_compiled(NPAD, g, K, W)) continue;
        if (exact_group_rows(deg.data(), NPAD, g, order.data())) { G = g; break; }
    }
    if (!G) return false;
    P->planes = K;
    P->words_tracked = W;
    P->ntracked = (int)tracked.size();
    P->npad = NPAD;
    P->G = G;
    P->NG = (NPAD + G - 1) / G;
    P->NL = P->NG + (NPAD > 32 ? 2 : 1);
    P->off_deg = align_up((size_t)NPAD * 8, 16);
    P->off_cm = align_up(P->off_deg + (size_t)NPAD * 4, 256);
    P->off_trm = align_up(P->off_cm + 64 * 8, 256);
    P->off_toff = align_up(P->off_trm + 64 * 8, 16);
    P->off_acc = align_up(P->off_toff + 64 * 4, 256);
    P->image.assign(P->off_acc, 0);
    uint64_t *rm = (uint64_t *)P->image.data();
    int32_t *dg = (int32_t *)(P->image.data() + P->off_deg);
    uint64_t *cm = (uint64_t *)(P->image.data() + P->off_cm);
    uint64_t *trm = (uint64_t *)(P->image.data() + P->off_trm);
    int32_t *toff = (int32_t *)(P->image.data() + P->off_toff);
    for (int i = 0; i < NPAD; i++) {
        rm[i] = rows[order[i]];
        dg[i] = (int32_t)deg[order[i]];
    }
    for (size_t e = 0; e < tracked.size(); e++) {
        const int r = tracked[e];
        trm[e] = rows[r];
        toff[e] = (int32_t)(deg[r] / 2);        // u = deg/2 - (ones in minus columns)
        for (int j = 0; j < n - 1; j++)
            if ((rows[r] >> j) & 1) cm[j] |= 1ull << e;
    }
    return true;
}

// One block sums the per-block slots of an exact or 0/1 launch into the
// result words (or takes the atomically added words, re-zeroing them) and
// moves the status out, re-arming it for the next launch.  Warp w sums words
// w, w + 8, ...; the slots are word-major, so a warp's loads coalesce.
__global__ void __launch_bounds__(256) exact_finish_kernel(const unsigned long long *part,
                                                           int blocks, int nl,
                                                           unsigned long long *acc, int *status,
                                                           unsigned long long *out,
                                                           unsigned long long *counter) {
#if EXACT_FINISH_PDL
    // launched as a programmatic dependent: wait for the walk grid's writes
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int l = warp; l < nl; l += nw) {
        long long t = 0;
        if (part) {
            for (int b = lane; b < blocks; b += 32) t += (long long)part[(size_t)l * blocks + b];
        } else if (lane == 0) {
            t = (long long)acc[l];
            acc[l] = 0;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
        if (lane == 0) out[l] = (unsigned long long)t;
    }
    if (threadIdx.x == 0) {
        out[nl] = (unsigned long long)(unsigned)*status;
        *status = 0;
        if (counter) *counter = 0;
    }
}

cudaError_t exact_finish(const unsigned long long *part, int blocks, int nl,
                         unsigned long long *acc, int *status, unsigned long long *out,
                         cudaStream_t stream, unsigned long long *counter) {
#if EXACT_FINISH_PDL
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, exact_finish_kernel, part, blocks, nl, acc, status, out,
                              counter);
#else
    exact_finish_kernel<<<1, 256, 0, stream>>>(part, blocks, nl, acc, status, out, counter);
    return cudaGetLastError();
#endif
}

// Per-block word slots after the result words (the kernels' epilogue);
// EXACT_BLOCK_SLOTS=0 makes the general kernel add into the shared words
// with atomics instead (for comparisons).
#ifndef EXACT_BLOCK_SLOTS
#define EXACT_BLOCK_SLOTS 1
#endif
static void add_block_slots(ExactPlan *P) {
    P->off_part = P->total;
    P->total = align_up(P->off_part + (size_t)P->blocks * P->NL * 8, 256);
    P->image.resize(P->total, 0);
}

static int plan_build(const int64_t *A, int n, ExactPlan *P) {
    if (plan_build_binary(A, n, P)) {
        DeviceInfo dev;
        int st = device_info(&dev);
        if (st != PG_OK) return st;
        st = abort_flag_device(&P->abort_dev);
        if (st != PG_OK) return st;
        P->n = n;
        P->need_bits = bound_bits(A, n) + 2;
        P->off_status = align_up(P->off_acc + (size_t)P->NL * 8, 256);
        P->off_out = align_up(P->off_status + 16, 256);
        P->total = align_up(P->off_out + (size_t)(P->NL + 1) * 8, 256);
        P->image.resize(P->total, 0);
        const int occ = occupancy_binary_any(P->npad, P->G, P->planes, P->words_tracked);
        uint64_t blocks = 0;
        int log_len = 0;
        exact_launch_shape(n - 1, occ, dev.sm_count, &blocks, &P->threads, &log_len);
        // chunks of 2^10 states (each starts from a closed-form tracker
        // state) while every thread still gets 16 of them round-robin
        const uint64_t T = blocks * (uint64_t)P->threads;
        while (log_len < 10 && ((1ull << (n - 1)) >> (log_len + 1)) >= 16 * T) log_len++;
        P->chunks.log_len = log_len;
        P->chunks.chunks = 1ull << (n - 1 - log_len);
        P->blocks = blocks;
        add_block_slots(P);
        return PG_OK;
    }
    std::vector<int> order;
    const int G = choose_group(A, n, &order);
    if (!G) return fail(PG_EOVERFLOW, "row-sum bound exceeds the exact engine's fixed widths");
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    st = abort_flag_device(&P->abort_dev);
    if (st != PG_OK) return st;
    const int N = n, NCOL = n - 1, NP = (n + 3) & ~3;
    const int fr_max = exact_frows_max(n, G);
    P->fr = exact_frows_arrange(A, n, G, fr_max, order.data()) ? fr_max : 0;
    P->n = n;
    P->G = G;
    P->NG = (N + G - 1) / G;
    P->NL = P->NG + (N > 32 ? 2 : 1);
    P->need_bits = bound_bits(A, n) + 2;
    const size_t off_init = align_up((size_t)NCOL * 2 * NP * 4, 256);
    P->off_acc = align_up(off_init + (size_t)NP * 4, 256);
    P->off_status = align_up(P->off_acc + (size_t)P->NL * 8, 256);
    P->off_out = align_up(P->off_status + 16, 256);
    P->total = align_up(P->off_out + (size_t)(P->NL + 1) * 8, 256);
    P->image.assign(P->total, 0);
    int32_t *tab = (int32_t *)P->image.data();
    int32_t *init = (int32_t *)(P->image.data() + off_init);
    for (int ii = 0; ii < N; ii++) {
        const int64_t *row = A + (size_t)order[ii] * n;
        const bool fl = P->fr > 0 && exact_float_row(N, G, P->fr, ii);
        const auto enc = [&](int64_t v) { return fl ? (int32_t)float_bits(v) : (int32_t)v; };
        int64_t sum = 0;
        for (int j = 0; j < n; j++) sum += row[j];
        init[ii] = enc(sum);
        for (int j = 0; j < NCOL; j++) {
            tab[(2 * j + 0) * NP + ii] = enc(2 * row[j]);
            tab[(2 * j + 1) * NP + ii] = enc(-2 * row[j]);
        }
    }
    // One resident wave of blocks (occupancy-limited), each thread owning a
    // contiguous range of chunks; short walks shrink the blocks, not the
    // number of SMs in use (exact_launch_shape).
    const int occ = P->fr ? occupancy_exact_frows(N, G, P->fr) : occupancy_exact_any(N, G);
    const int log_states = n - 1;
    uint64_t blocks = 0;
    int log_len = 0;
    exact_launch_shape(log_states, occ, dev.sm_count, &blocks, &P->threads, &log_len);
    P->chunks.log_len = log_len;
    P->chunks.chunks = 1ull << (log_states - log_len);
    P->blocks = blocks;
    add_block_slots(P);
    return PG_OK;
}

// Upload tables and zero the accumulators, status and result words
// (async on P->stream).  Launches re-zero what they use, so this runs once
// per plan.
static int plan_upload(ExactPlan *P) {
    std::memcpy(P->host, P->image.data(), P->total);
    PG_CUDA(cudaMemcpyAsync(P->dev, P->host, P->off_acc, cudaMemcpyHostToDevice, P->stream));
    PG_CUDA(cudaMemsetAsync(P->dev + P->off_acc, 0, P->total - P->off_acc, P->stream));
    return PG_OK;
}

// One launch (async on `stream`): the kernel and its one-block finisher,
// no memset.
static int plan_launch(ExactPlan *P, cudaStream_t stream) {
    if (P->planes) {
        BinaryArgs b;
        b.rmask = (const uint64_t *)P->dev;
        b.deg = (const int32_t *)(P->dev + P->off_deg);
        b.cmask = (const uint64_t *)(P->dev + P->off_cm);
        b.trmask = (const uint64_t *)(P->dev + P->off_trm);
        b.toff = (const int32_t *)(P->dev + P->off_toff);
        b.ntracked = P->ntracked;
        b.n = P->n;
        b.acc = (unsigned long long *)(P->dev + P->off_acc);
        b.status = (int *)(P->dev + P->off_status);
        b.part = (unsigned long long *)(P->dev + P->off_part);
        // the chunk-group counter of the split instantiation shares the
        // status slot's second 8 bytes
        b.next = (unsigned long long *)(P->dev + P->off_status + 8);
        b.abort_flag = P->abort_dev;
        b.chunks = P->chunks.chunks;
        b.log_len = P->chunks.log_len;
        b.chunk0 = P->chunk0;
        b.threads = P->threads;
        // evaluation from the warp's common high Gray bits: the window must
        // start on a multiple of 32 chunks
        const bool split = P->bin_split && (P->chunk0 & 31) == 0 && P->chunks.log_len + 5 <= 31;
        PG_CUDA(launch_binary_any(P->npad, P->G, P->planes, P->words_tracked, b, split,
                                  (int)P->blocks, stream));
        PG_CUDA(exact_finish(b.part, (int)P->blocks, P->NL, b.acc, b.status,
                             (unsigned long long *)(P->dev + P->off_out), stream,
                             split ? b.next : nullptr));
        return PG_OK;
    }
    ExactArgs args;
    args.tab = (const int32_t *)P->dev;
    args.init = (const int32_t *)(P->dev + align_up((size_t)(P->n - 1) * 2 * ((P->n + 3) & ~3) * 4, 256));
    args.acc = (unsigned long long *)(P->dev + P->off_acc);
    args.status = (int *)(P->dev + P->off_status);
    args.abort_flag = P->abort_dev;
    args.chunks = P->chunks.chunks;
    args.log_len = P->chunks.log_len;
    args.chunk0 = P->chunk0;
    args.threads = P->threads;
    args.part = EXACT_BLOCK_SLOTS ? (unsigned long long *)(P->dev + P->off_part) : nullptr;
    PG_CUDA(P->fr ? launch_exact_frows(P->n, P->G, P->fr, args, (int)P->blocks, stream)
                  : launch_exact_any(P->n, P->G, args, (int)P->blocks, stream));
    PG_CUDA(exact_finish(args.part, (int)P->blocks, P->NL, args.acc, args.status,
                         (unsigned long long *)(P->dev + P->off_out), stream));
    return PG_OK;
}

// Restrict a built plan to Gray states [lo, hi): both must be multiples of
// 4 (the kernel's two-step unroll keeps chunk starts even and aligned).
static int plan_restrict(ExactPlan *P, uint64_t lo, uint64_t hi) {
    const uint64_t states = 1ull << (P->n - 1);
    if (lo >= hi || hi > states) return fail(PG_ERANGE, "state range must satisfy lo < hi <= 2^(n-1)");
    int ll = P->chunks.log_len;
    while (ll > 0 && (((lo | hi) & ((1ull << ll) - 1)) != 0)) ll--;
    const int logu = (P->n - 1) < EXACT_LOGU ? (P->n - 1) : EXACT_LOGU;
    if (ll < logu || ll < 1)
        return fail(PG_EINVAL, "state range bounds must be multiples of 4");
    P->chunks.log_len = ll;
    P->chunk0 = lo >> ll;
    P->chunks.chunks = (hi - lo) >> ll;
    return PG_OK;
}

// Copy the accumulators back (sync) and carry them into per(A).
static int plan_finish(ExactPlan *P, cudaStream_t stream, uint32_t *out, int limbs) {
    if (32 * limbs < P->need_bits)
        return fail(PG_ERANGE, "output limb count too small for the permanent bound");
    const int NL = P->NL, W = NL + 3;
    PG_CUDA(cudaMemcpyAsync(P->host + P->off_out, P->dev + P->off_out, (size_t)(NL + 1) * 8,
                            cudaMemcpyDeviceToHost, stream));
    PG_CUDA(cudaStreamSynchronize(stream));
    const long long *acc = (const long long *)(P->host + P->off_out);
    if (acc[NL]) return fail(PG_EABORT, "exact launch aborted by pg_abort()");
    std::vector<uint32_t> S(W, 0);
    for (int l = 0; l < NL; l++) add_i64_at(S, l, acc[l]);
    const int sh = P->n - 1;
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

int exact_run(const int64_t *A, int n, uint32_t *out, int limbs) {
    ExactPlan P;
    int st = plan_build(A, n, &P);
    if (st != PG_OK) return st;
    if (32 * limbs < P.need_bits)
        return fail(PG_ERANGE, "output limb count too small for the permanent bound");
    Workspace *ws;
    st = workspace(&ws, P.total, P.total);
    if (st != PG_OK) return st;
    P.dev = (char *)ws->dev;
    P.host = (char *)ws->host;
    P.stream = ws->stream;
    if ((st = plan_upload(&P)) != PG_OK) return st;
    if ((st = plan_launch(&P, P.stream)) != PG_OK) return st;
    return plan_finish(&P, P.stream, out, limbs);
}

}  // namespace pg

struct pg_exact_plan {
    pg::ExactPlan p;
};

extern "C" {

int pg_exact_supported(const int64_t *A, int n) {
    if (!A || n < 2 || n > 48) return 0;
    std::vector<int> order;
    return pg::choose_group(A, n, &order) ? 1 : 0;
}

int pg_exact_permanent(const int64_t *A, int n, uint32_t *out, int limbs) {
    using namespace pg;
    if (n < 0 || n >= 64) return fail(PG_ERANGE, "matrix dimension must be less than 64");
    if (limbs < 1 || !out) return fail(PG_EINVAL, "out/limbs invalid");
    if (n > 0 && !A) return fail(PG_EINVAL, "matrix is null");
    if (n <= 1) {
        const int64_t v = n == 0 ? 1 : A[0];
        if (limbs == 1 && (v < INT32_MIN || v > INT32_MAX))
            return fail(PG_ERANGE, "output limb count too small");
        for (int i = 0; i < limbs; i++)
            out[i] = i == 0 ? (uint32_t)(uint64_t)v
                   : i == 1 ? (uint32_t)((uint64_t)v >> 32)
                   : (v < 0 ? 0xffffffffu : 0u);
        return PG_OK;
    }
    return exact_run(A, n, out, limbs);
}

int pg_exact_partial(const int64_t *A, int n, uint64_t state_lo, uint64_t state_hi,
                     int64_t *words, int max_words, int *nwords) {
    using namespace pg;
    if (!A || !words || !nwords || n < 2 || n >= 64) return fail(PG_EINVAL, "bad arguments");
    ExactPlan P;
    int st = plan_build(A, n, &P);
    if (st != PG_OK) return st;
    if ((st = plan_restrict(&P, state_lo, state_hi)) != PG_OK) return st;
    if (max_words < P.NL) return fail(PG_ERANGE, "words buffer too small");
    Workspace *ws;
    st = workspace(&ws, P.total, P.total);
    if (st != PG_OK) return st;
    P.dev = (char *)ws->dev;
    P.host = (char *)ws->host;
    P.stream = ws->stream;
    if ((st = plan_upload(&P)) != PG_OK) return st;
    if ((st = plan_launch(&P, P.stream)) != PG_OK) return st;
    PG_CUDA(cudaMemcpyAsync(P.host + P.off_out, P.dev + P.off_out, (size_t)(P.NL + 1) * 8,
                            cudaMemcpyDeviceToHost, P.stream));
    PG_CUDA(cudaStreamSynchronize(P.stream));
    if (((const long long *)(P.host + P.off_out))[P.NL])
        return fail(PG_EABORT, "aborted by pg_abort()");
    std::memcpy(words, P.host + P.off_out, (size_t)P.NL * 8);
    *nwords = P.NL;
    return PG_OK;
}

int pg_exact_plan_create(const int64_t *A, int n, pg_exact_plan **out) {
    using namespace pg;
    if (!out) return fail(PG_EINVAL, "out is null");
    *out = nullptr;
    if (n < 2 || n >= 64 || !A) return fail(PG_ERANGE, "plans need 2 <= n < 64 and a matrix");
    pg_exact_plan *h = new pg_exact_plan();
    int st = plan_build(A, n, &h->p);
    if (st != PG_OK) { delete h; return st; }
    ExactPlan &P = h->p;
    cudaError_t e = cudaMalloc((void **)&P.dev, P.total);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&P.host, P.total, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking);
    P.owns = true;
    if (e != cudaSuccess) {
        st = cuda_fail(e, "pg_exact_plan_create");
        pg_exact_plan_destroy(h);
        return st;
    }
    st = plan_upload(&P);
    if (st == PG_OK) {
        e = cudaStreamSynchronize(P.stream);
        if (e != cudaSuccess) st = cuda_fail(e, "pg_exact_plan_create");
    }
    if (st != PG_OK) { pg_exact_plan_destroy(h); return st; }
    *out = h;
    return PG_OK;
}

int pg_exact_plan_launch(pg_exact_plan *plan, void *stream) {
    using namespace pg;
    if (!plan) return fail(PG_EINVAL, "plan is null");
    return plan_launch(&plan->p, stream ? (cudaStream_t)stream : plan->p.stream);
}

int pg_exact_plan_result(pg_exact_plan *plan, void *stream, uint32_t *out, int limbs) {
    using namespace pg;
    if (!plan || !out || limbs < 1) return fail(PG_EINVAL, "null argument");
    return plan_finish(&plan->p, stream ? (cudaStream_t)stream : plan->p.stream, out, limbs);
}

int pg_exact_plan_info(const pg_exact_plan *plan, int *group, int *words,
                       uint64_t *states, uint64_t *imul_per_state,
                       uint64_t *imad_wide_per_state) {
    using namespace pg;
    if (!plan) return fail(PG_EINVAL, "plan is null");
    const ExactPlan &P = plan->p;
    if (group) *group = P.G;
    if (words) *words = P.NG;
    if (states) *states = 1ull << (P.n - 1);
    // the algorithm's row-group multiplies (with float rows most of them
    // run as exact FP32 multiplies on the FP32 pipe)
    if (imul_per_state) *imul_per_state = (uint64_t)(P.n - P.NG);
    if (imad_wide_per_state) *imad_wide_per_state = (uint64_t)P.NG * (P.NG - 1) / 2;
    return PG_OK;
}

int pg_exact_plan_float_rows(const pg_exact_plan *plan) {
    return plan ? plan->p.fr : 0;
}

int pg_exact_plan_bit_planes(const pg_exact_plan *plan) {
    return plan ? plan->p.planes : 0;
}

void pg_exact_plan_destroy(pg_exact_plan *plan) {
    if (!plan) return;
    pg::ExactPlan &P = plan->p;
    if (P.owns) {
        if (P.stream) cudaStreamSynchronize(P.stream);
        if (P.dev) cudaFree(P.dev);
        if (P.host) cudaFreeHost(P.host);
        if (P.stream) cudaStreamDestroy(P.stream);
    }
    delete plan;
}

}  // extern "C"
