// Batched exact Glynn engine: thousands of integer matrices of uneven order
// in one persistent, work-stealing launch captured in a CUDA graph.
//
// Work unit ("task"): 32 lanes x k chunks of one matrix; lane l walks chunks
// [c0 + l*k, c0 + (l+1)*k), so all lanes share the chunk-local Gray columns
// and the matrix's column table, staged per warp in shared memory.  Warps
// take tasks from a global atomic counter; the host orders tasks by
// decreasing work (largest orders first) so the tail is made of small
// tasks.  Each task's per-word sums are warp-reduced and added to the
// matrix's 64-bit words with one atomic per word.  Orders 2..32 are compiled
// (row groups of 4, and of 5 from order 20: batch_compiled); matrices outside that
// range or whose groups do not fit are evaluated by the single-matrix exact
// engine when the results are collected.
//
// Tuning knobs (pg_batch_tune): log2 states per lane per task, blocks per
// SM, chunk length.  permgpu.autotune searches them and persists the best.
#include "pg_internal.h"
#include "exact_glynn.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace pg {

int exact_run(const int64_t *A, int n, uint32_t *out, int limbs);

static constexpr int BATCH_MAX_N = 32;
static constexpr int BATCH_NP = 32;                  // row stride in the per-warp slice
static constexpr int BATCH_SLICE = (BATCH_MAX_N - 1) * 2 * BATCH_NP + BATCH_NP;  // int32 per warp
static constexpr int BATCH_WORDS = 10;               // accumulator words per matrix

struct BatchTask {
    uint32_t m;      // matrix index
    uint32_t k;      // chunks per lane
    uint64_t c0;     // first chunk of lane 0
};

struct BatchArgs {
    const int32_t *tables;        // concatenated [tab | init] per matrix
    const uint64_t *table_off;    // int32 offset of each matrix's table
    const uint8_t *orders;        // n per matrix
    const uint8_t *groups;        // row-group size G per matrix
    const uint8_t *frows;         // float rows per group (0 or 3) per matrix
    const uint8_t *log_len;       // chunk log length per matrix
    const uint64_t *chunks;       // chunks per matrix
    const BatchTask *tasks;
    uint32_t ntasks;
    unsigned int *counter;        // zeroed per launch
    unsigned long long *acc;      // [count][BATCH_WORDS]
    int *status;
    volatile const int *abort_flag;
};

// Group sizes compiled into the batch kernel: 4 (N < 4: N) for every order
// and 5 for orders 20..32, where the time of a batch goes; the host takes
// the largest whose groups fit (small entries: fewer product words per term).
__host__ __device__ constexpr bool batch_compiled(int N, int G) {
    return N < 2 || N > BATCH_MAX_N ? false
           : N < 4 ? G == N
           : G == 4 || (G == 5 && N >= 20);
}
// Float rows (exact_glynn.cuh): three of each group's rows as exact FP32
// sums, so a group of 4 costs one IMUL instead of three.  Compiled for
// groups of 4 at orders 20, 24 and 28 (where the batch's time goes); a
// matrix of order 21..27 whose rows qualify runs at the next of these
// orders with constant rows s = 1 added (zero table entries), which leaves
// its walk, its permanent and its product words unchanged.  Other float-row
// shapes made the shared kernel spill.
__host__ __device__ constexpr bool batch_frows_compiled(int N, int G) {
    return (N == 20 || N == 24 || N == 28) && G == 4;
}
constexpr int BATCH_FROWS = 3;
// 1: a matrix whose rows fit groups of 5 takes groups of 4 with float rows
// instead.  Measured on batch4096 (entries in [-3, 3]): 313 ms against
// 264 ms with groups of 5, so the default keeps groups of 5.
#ifndef BATCH_FROWS_FIRST
#define BATCH_FROWS_FIRST 0
#endif
__host__ __device__ constexpr int batch_frows_order(int n) {
    return n >= 20 && n <= 28 ? (n + 3) & ~3 : 0;
}

template <int N, int G, int FR = 0>
__device__ __forceinline__ void batch_task(const int32_t *wtab, const BatchArgs &a,
                                           const BatchTask &t, int lane) {
    using S = ExactShape<N, G>;
    constexpr int NP = S::NP, NL = S::NL;
    // the warp slice stores rows with stride BATCH_NP; exact_walk indexes
    // with NP, so the host packs each table with stride NP inside the slice
    const int log_len = a.log_len[t.m];
    const uint64_t nch = a.chunks[t.m];
    uint64_t cb = t.c0 + (uint64_t)lane * t.k;
    uint64_t ce = cb + t.k;
    if (cb > nch) cb = nch;
    if (ce > nch) ce = nch;
    uint32_t acc[NL];
#pragma unroll
    for (int l = 0; l < NL; l++) acc[l] = 0;
    bool ok = true;
    if (cb < ce) {
        int32_t s[N];
        exact_init<N, G, FR>(wtab, wtab + (N - 1) * 2 * NP, s, cb << log_len);
        ok = exact_walk<N, G, FR>(wtab, s, acc, cb, ce, log_len, a.abort_flag);
    }
    if (!ok) atomicExch(a.status, 1);
#pragma unroll
    for (int l = 0; l < NL; l++) {
        long long v = (l == NL - 1) ? (long long)(int32_t)acc[l] : (long long)acc[l];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0 && v != 0)
            atomicAdd(a.acc + (size_t)t.m * BATCH_WORDS + l, (unsigned long long)v);
    }
}

__global__ void __launch_bounds__(256, 2) batch_glynn_kernel(BatchArgs a) {
    extern __shared__ int4 bsmem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t *wtab = reinterpret_cast<int32_t *>(bsmem) + warp * BATCH_SLICE;
    uint32_t cur = 0xffffffffu;
    for (unsigned int k = 0;; k++) {
        // the host-mapped abort word, once per 8 tasks of the warp (a task's
        // own walk reads it only past 2^16 states per lane)
        if (k != 0 && (k & 7) == 0 && __any_sync(0xffffffffu, *a.abort_flag != 0)) {
            if (lane == 0) atomicExch(a.status, 1);
            break;
        }
        unsigned int ti = 0;
        if (lane == 0) ti = atomicAdd(a.counter, 1u);
        ti = __shfl_sync(0xffffffffu, ti, 0);
        if (ti >= a.ntasks) break;
        const BatchTask t = a.tasks[ti];
        const int n = a.orders[t.m];
        if (t.m != cur) {
            const int NP = (n + 3) & ~3;
            const int words = (n - 1) * 2 * NP + NP;
            const int32_t *src = a.tables + a.table_off[t.m];
            __syncwarp();
            for (int i = lane; i < words; i += 32) wtab[i] = __ldg(src + i);
            __syncwarp();
            cur = t.m;
        }
        switch (n * 16 + a.groups[t.m] * 2 + (a.frows[t.m] ? 1 : 0)) {
#define PG_BATCH_CASE(NN, GG) \
    case NN * 16 + GG * 2: batch_task<NN, GG>(wtab, a, t, lane); break;
#define PG_BATCH_FCASE(NN, GG) \
    case NN * 16 + GG * 2 + 1: batch_task<NN, GG, BATCH_FROWS>(wtab, a, t, lane); break;
            PG_BATCH_CASE(2, 2) PG_BATCH_CASE(3, 3)
#define PG_BATCH_G4(NN) PG_BATCH_CASE(NN, 4)
#define PG_BATCH_G5(NN) PG_BATCH_CASE(NN, 5)
            PG_BATCH_G4(4) PG_BATCH_G4(5) PG_BATCH_G4(6) PG_BATCH_G4(7) PG_BATCH_G4(8)
            PG_BATCH_G4(9) PG_BATCH_G4(10) PG_BATCH_G4(11) PG_BATCH_G4(12) PG_BATCH_G4(13)
            PG_BATCH_G4(14) PG_BATCH_G4(15) PG_BATCH_G4(16) PG_BATCH_G4(17) PG_BATCH_G4(18)
            PG_BATCH_G4(19) PG_BATCH_G4(20) PG_BATCH_G4(21) PG_BATCH_G4(22) PG_BATCH_G4(23)
            PG_BATCH_G4(24) PG_BATCH_G4(25) PG_BATCH_G4(26) PG_BATCH_G4(27) PG_BATCH_G4(28)
            PG_BATCH_G4(29) PG_BATCH_G4(30) PG_BATCH_G4(31) PG_BATCH_G4(32)
            PG_BATCH_G5(20)
            PG_BATCH_G5(21) PG_BATCH_G5(22) PG_BATCH_G5(23) PG_BATCH_G5(24) PG_BATCH_G5(25)
            PG_BATCH_G5(26) PG_BATCH_G5(27) PG_BATCH_G5(28) PG_BATCH_G5(29) PG_BATCH_G5(30)
            PG_BATCH_G5(31) PG_BATCH_G5(32)
#define PG_BATCH_F(NN) PG_BATCH_FCASE(NN, 4)
            PG_BATCH_F(20) PG_BATCH_F(24) PG_BATCH_F(28)
#undef PG_BATCH_F
#undef PG_BATCH_G4
#undef PG_BATCH_G5
#undef PG_BATCH_FCASE
#undef PG_BATCH_CASE
        default: break;
        }
    }
}

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

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

// Row order for the largest compiled group size whose groups fit
// (exact_group_rows); returns that size, or 0.
static int batch_group(const int64_t *A, int n, std::vector<int> *order) {
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
    for (int G = 5; G >= 2; G--)
        if (batch_compiled(n, G) && exact_group_rows(B.data(), n, G, order->data())) return G;
    return 0;
}

struct BatchPlan {
    int count = 0;
    std::vector<int> orders;
    std::vector<uint8_t> groups;           // row-group size of each kernel matrix
    std::vector<uint8_t> frows;            // float rows per group (0 or 3)
    std::vector<uint8_t> korder;           // order the kernel runs (padded for float rows)
    std::vector<uint8_t> in_kernel;        // 1 if the batch kernel evaluates it
    std::vector<std::vector<int64_t>> external;  // matrices for the single engine
    std::vector<int> ext_index;
    std::vector<double> bound_bits;
    size_t total = 0, off_acc = 0, off_counter = 0, off_status = 0;
    uint32_t ntasks = 0;
    int blocks = 0;
    size_t smem = 0;
    char *dev = nullptr;
    char *host = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    BatchArgs args{};
    uint64_t kernel_states = 0;
};

}  // namespace pg

struct pg_batch_plan {
    pg::BatchPlan p;
};

extern "C" {

int pg_batch_plan_create(const int64_t *A, const int64_t *offsets, const int32_t *orders,
                         int count, const pg_batch_tune *tune, pg_batch_plan **out) {
    using namespace pg;
    if (!out) return fail(PG_EINVAL, "out is null");
    *out = nullptr;
    if (count < 0 || (count > 0 && (!A || !offsets || !orders)))
        return fail(PG_EINVAL, "batch arguments invalid");
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;

    const int lane_log = tune && tune->lane_log_states > 0 ? tune->lane_log_states : 13;
    const int chunk_log = tune && tune->chunk_log_len > 0 ? tune->chunk_log_len : 6;
    const int bps = tune && tune->blocks_per_sm > 0 ? tune->blocks_per_sm : 2;

    pg_batch_plan *h = new pg_batch_plan();
    BatchPlan &P = h->p;
    P.count = count;
    P.orders.assign(orders, orders + count);
    P.in_kernel.assign(count, 0);
    P.groups.assign(count, 0);
    P.frows.assign(count, 0);
    P.korder.assign(count, 0);
    P.ext_index.assign(count, -1);
    P.bound_bits.assign(count, 0.0);

    std::vector<int32_t> tables;
    std::vector<uint64_t> toff(count, 0), nchunks(count, 0);
    std::vector<uint8_t> ord8(count, 0), loglen(count, 0);
    std::vector<BatchTask> tasks;
    std::vector<uint64_t> task_work;
    for (int m = 0; m < count; m++) {
        const int n = orders[m];
        if (n < 0 || n >= 64) { delete h; return fail(PG_ERANGE, "matrix order must be 0 <= n < 64"); }
        const int64_t *a = A + offsets[m];
        double bits = 0;
        for (int i = 0; i < n; i++) {
            double rs = 0;
            for (int j = 0; j < n; j++) rs += std::fabs((double)a[(size_t)i * n + j]);
            bits += std::log2(rs < 1 ? 1 : rs);
        }
        P.bound_bits[m] = bits;
        std::vector<int> order;
        int G = n < 2 || n > BATCH_MAX_N ? 0 : batch_group(a, n, &order);
        if (!G) {
            P.ext_index[m] = (int)P.external.size();
            P.external.emplace_back(a, a + (size_t)n * n);
            continue;
        }
        P.in_kernel[m] = 1;
        // float rows at the padded order K: a bound-only K x K image whose
        // extra rows have bound 1 picks the grouping and the float rows
        int K = n, FR = 0;
        const int KF = batch_frows_order(n);
        if ((G == 4 || (BATCH_FROWS_FIRST && G == 5)) && batch_frows_compiled(KF, 4)) {
            std::vector<int64_t> img((size_t)KF * KF, 0);
            for (int i = 0; i < KF; i++)
                for (int j = 0; j < KF; j++)
                    img[(size_t)i * KF + j] = i < n ? (j < n ? a[(size_t)i * n + j] : 0) : (j == 0);
            std::vector<uint64_t> Bk(KF);
            for (int i = 0; i < KF; i++) {
                uint64_t b = 0;
                for (int j = 0; j < KF; j++) b += (uint64_t)std::llabs(img[(size_t)i * KF + j]);
                Bk[i] = b;
            }
            std::vector<int> ko(KF);
            if (exact_group_rows(Bk.data(), KF, 4, ko.data()) &&
                exact_frows_arrange(img.data(), KF, 4, BATCH_FROWS, ko.data())) {
                K = KF;
                FR = BATCH_FROWS;
                G = 4;
                order = ko;
            }
        }
        P.groups[m] = (uint8_t)G;
        P.frows[m] = (uint8_t)FR;
        P.korder[m] = (uint8_t)K;
        const int NP = (K + 3) & ~3;
        toff[m] = tables.size();
        const size_t base = tables.size();
        tables.resize(base + (size_t)(K - 1) * 2 * NP + NP, 0);
        for (int ii = 0; ii < K; ii++) {
            const bool fl = FR > 0 && exact_float_row(K, G, FR, ii);
            const auto enc = [&](int64_t v) {
                return fl ? (int32_t)exact_float_bits((float)v) : (int32_t)v;
            };
            if (order[ii] >= n) {          // added constant row: s = 1, no column
                tables[base + (size_t)(K - 1) * 2 * NP + ii] = enc(1);
                continue;
            }
            const int64_t *row = a + (size_t)order[ii] * n;
            int64_t sum = 0;
            for (int j = 0; j < n; j++) sum += row[j];
            tables[base + (size_t)(K - 1) * 2 * NP + ii] = enc(sum);
            for (int j = 0; j < n - 1; j++) {
                tables[base + (size_t)(2 * j + 0) * NP + ii] = enc(2 * row[j]);
                tables[base + (size_t)(2 * j + 1) * NP + ii] = enc(-2 * row[j]);
            }
        }
        const int log_states = n - 1;
        const int LOGU = log_states < EXACT_LOGU ? log_states : EXACT_LOGU;
        int ll = chunk_log < log_states ? chunk_log : log_states;
        if (ll < LOGU) ll = LOGU;
        if (ll < 1) ll = 1;
        const uint64_t ch = 1ull << (log_states - ll);
        uint64_t k = lane_log > ll ? (1ull << (lane_log - ll)) : 1;
        if (k * 32 > ch) k = (ch + 31) / 32;
        if (k < 1) k = 1;
        ord8[m] = (uint8_t)K;
        loglen[m] = (uint8_t)ll;
        nchunks[m] = ch;
        P.kernel_states += 1ull << log_states;
        for (uint64_t c0 = 0; c0 < ch; c0 += 32 * k) {
            tasks.push_back(BatchTask{(uint32_t)m, (uint32_t)k, c0});
            const uint64_t span = std::min<uint64_t>(32 * k, ch - c0);
            // cost model: states of the busiest lane times per-state work ~ n
            task_work.push_back(std::min<uint64_t>(k, span) * (1ull << ll) * (uint64_t)n);
        }
    }
    // largest tasks first (LPT order); ties keep matrix order
    std::vector<uint32_t> idx(tasks.size());
    for (size_t i = 0; i < idx.size(); i++) idx[i] = (uint32_t)i;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](uint32_t x, uint32_t y) { return task_work[x] > task_work[y]; });
    std::vector<BatchTask> sorted(tasks.size());
    for (size_t i = 0; i < idx.size(); i++) sorted[i] = tasks[idx[i]];
    P.ntasks = (uint32_t)sorted.size();

    const size_t off_tables = 0;
    const size_t off_toff = align_up(off_tables + tables.size() * 4, 256);
    const size_t off_ord = align_up(off_toff + (size_t)count * 8, 256);
    const size_t off_grp = align_up(off_ord + (size_t)count, 256);
    const size_t off_fr = align_up(off_grp + (size_t)count, 256);
    const size_t off_ll = align_up(off_fr + (size_t)count, 256);
    const size_t off_nch = align_up(off_ll + (size_t)count, 256);
    const size_t off_tasks = align_up(off_nch + (size_t)count * 8, 256);
    P.off_acc = align_up(off_tasks + sorted.size() * sizeof(BatchTask), 256);
    P.off_counter = align_up(P.off_acc + (size_t)count * BATCH_WORDS * 8, 256);
    P.off_status = P.off_counter + 64;
    P.total = align_up(P.off_status + 64, 256);

    cudaError_t e = cudaMalloc((void **)&P.dev, P.total);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&P.host, P.total, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        st = cuda_fail(e, "pg_batch_plan_create");
        pg_batch_plan_destroy(h);
        return st;
    }
    std::memset(P.host, 0, P.total);
    if (!tables.empty()) std::memcpy(P.host + off_tables, tables.data(), tables.size() * 4);
    std::memcpy(P.host + off_toff, toff.data(), (size_t)count * 8);
    std::memcpy(P.host + off_ord, ord8.data(), (size_t)count);
    if (count) std::memcpy(P.host + off_grp, P.groups.data(), (size_t)count);
    if (count) std::memcpy(P.host + off_fr, P.frows.data(), (size_t)count);
    std::memcpy(P.host + off_ll, loglen.data(), (size_t)count);
    std::memcpy(P.host + off_nch, nchunks.data(), (size_t)count * 8);
    if (!sorted.empty())
        std::memcpy(P.host + off_tasks, sorted.data(), sorted.size() * sizeof(BatchTask));
    e = cudaMemcpyAsync(P.dev, P.host, P.off_acc, cudaMemcpyHostToDevice, P.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(P.stream);
    if (e != cudaSuccess) {
        st = cuda_fail(e, "pg_batch_plan_create upload");
        pg_batch_plan_destroy(h);
        return st;
    }

    BatchArgs &a = P.args;
    a.tables = (const int32_t *)(P.dev + off_tables);
    a.table_off = (const uint64_t *)(P.dev + off_toff);
    a.orders = (const uint8_t *)(P.dev + off_ord);
    a.groups = (const uint8_t *)(P.dev + off_grp);
    a.frows = (const uint8_t *)(P.dev + off_fr);
    a.log_len = (const uint8_t *)(P.dev + off_ll);
    a.chunks = (const uint64_t *)(P.dev + off_nch);
    a.tasks = (const BatchTask *)(P.dev + off_tasks);
    a.ntasks = P.ntasks;
    a.counter = (unsigned int *)(P.dev + P.off_counter);
    a.acc = (unsigned long long *)(P.dev + P.off_acc);
    a.status = (int *)(P.dev + P.off_status);
    a.abort_flag = abort_dev;

    P.smem = (size_t)8 * BATCH_SLICE * sizeof(int32_t);
    e = cudaFuncSetAttribute(batch_glynn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)P.smem);
    int occ = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_glynn_kernel, 256, P.smem);
    if (e != cudaSuccess) {
        st = cuda_fail(e, "batch kernel attributes");
        pg_batch_plan_destroy(h);
        return st;
    }
    P.blocks = dev.sm_count * std::max(1, std::min(occ, bps));

    // Capture [zero accumulators/counter/status, persistent kernel] once.
    e = cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaMemsetAsync(P.dev + P.off_acc, 0, P.total - P.off_acc, P.stream);
        if (P.ntasks)
            batch_glynn_kernel<<<P.blocks, 256, P.smem, P.stream>>>(a);
        e = cudaStreamEndCapture(P.stream, &P.graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&P.exec, P.graph, 0);
    if (e != cudaSuccess) {
        st = cuda_fail(e, "batch graph capture");
        pg_batch_plan_destroy(h);
        return st;
    }
    *out = h;
    return PG_OK;
}

int pg_batch_plan_launch(pg_batch_plan *plan, void *stream) {
    using namespace pg;
    if (!plan) return fail(PG_EINVAL, "plan is null");
    PG_CUDA(cudaGraphLaunch(plan->p.exec, stream ? (cudaStream_t)stream : plan->p.stream));
    return PG_OK;
}

int pg_batch_plan_result(pg_batch_plan *plan, void *stream, uint32_t *out, int limbs) {
    using namespace pg;
    if (!plan || !out || limbs < 1) return fail(PG_EINVAL, "null argument");
    BatchPlan &P = plan->p;
    cudaStream_t s = stream ? (cudaStream_t)stream : P.stream;
    for (int m = 0; m < P.count; m++)
        if (P.bound_bits[m] + 2 > 32.0 * limbs)
            return fail(PG_ERANGE, "limbs per matrix too small for a matrix's bound");
    PG_CUDA(cudaMemcpyAsync(P.host + P.off_acc, P.dev + P.off_acc, P.total - P.off_acc,
                            cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    if (*(int *)(P.host + P.off_status))
        return fail(PG_EABORT, "batch launch aborted by pg_abort()");
    const long long *acc = (const long long *)(P.host + P.off_acc);
    for (int m = 0; m < P.count; m++) {
        uint32_t *o = out + (size_t)m * limbs;
        const int n = P.orders[m];
        if (!P.in_kernel[m]) {
            const std::vector<int64_t> &a = P.external[P.ext_index[m]];
            int st = pg_exact_permanent(a.data(), n, o, limbs);
            if (st != PG_OK) return st;
            continue;
        }
        const int W = BATCH_WORDS + 3;
        std::vector<uint32_t> S(W, 0);
        const int G = P.groups[m];
        const int NL = (P.korder[m] + G - 1) / G + 1;   // words of the order the kernel ran
        for (int l = 0; l < NL; l++) add_i64_at(S, l, acc[(size_t)m * BATCH_WORDS + l]);
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
            o[i] = bo ? (lo >> bo) | (hi << (32 - bo)) : lo;
        }
    }
    return PG_OK;
}

int pg_batch_plan_info(const pg_batch_plan *plan, uint32_t *tasks, int *blocks,
                       uint64_t *kernel_states, int *external) {
    using namespace pg;
    if (!plan) return fail(PG_EINVAL, "plan is null");
    if (tasks) *tasks = plan->p.ntasks;
    if (blocks) *blocks = plan->p.blocks;
    if (kernel_states) *kernel_states = plan->p.kernel_states;
    if (external) *external = (int)plan->p.external.size();
    return PG_OK;
}

void pg_batch_plan_destroy(pg_batch_plan *plan) {
    if (!plan) return;
    pg::BatchPlan &P = plan->p;
    if (P.stream) cudaStreamSynchronize(P.stream);
    if (P.exec) cudaGraphExecDestroy(P.exec);
    if (P.graph) cudaGraphDestroy(P.graph);
    if (P.dev) cudaFree(P.dev);
    if (P.host) cudaFreeHost(P.host);
    if (P.stream) cudaStreamDestroy(P.stream);
    delete plan;
}

int pg_batch_exact(const int64_t *A, const int64_t *offsets, const int32_t *orders,
                   int count, uint32_t *out, int limbs) {
    pg_batch_plan *plan = nullptr;
    int st = pg_batch_plan_create(A, offsets, orders, count, nullptr, &plan);
    if (st != PG_OK) return st;
    st = pg_batch_plan_launch(plan, nullptr);
    if (st == PG_OK) st = pg_batch_plan_result(plan, nullptr, out, limbs);
    pg_batch_plan_destroy(plan);
    return st;
}

// Residues of many matrices, each modulo its own list of moduli.  Matrices
// the exact engine accepts go through one batched exact launch and their
// exact values are reduced on the host; the others (entries too large for
// exact int32 row sums) take pg_residues, all of a matrix's moduli in one
// launch.
int pg_batch_residues(const int64_t *A, const int64_t *offsets, const int32_t *orders,
                      int count, const uint64_t *moduli, const int32_t *moduli_offsets,
                      uint64_t *out) {
    using namespace pg;
    if (count < 0) return fail(PG_EINVAL, "count must be non-negative");
    if (count == 0) return PG_OK;
    if (!A || !offsets || !orders || !moduli || !moduli_offsets || !out)
        return fail(PG_EINVAL, "null argument");
    for (int m = 0; m < count; m++) {
        if (orders[m] < 0 || orders[m] >= 64) return fail(PG_ERANGE, "orders must be < 64");
        if (moduli_offsets[m + 1] < moduli_offsets[m]) return fail(PG_EINVAL, "moduli offsets");
        for (int t = moduli_offsets[m]; t < moduli_offsets[m + 1]; t++)
            if (moduli[t] == 0 || moduli[t] >= (1ull << 63))
                return fail(PG_ERANGE, "moduli must satisfy 1 <= m < 2^63");
    }
    std::vector<int> exact_ids;
    std::vector<int64_t> packed, poff;
    std::vector<int32_t> pord;
    int limbs = 2;
    for (int m = 0; m < count; m++) {
        const int n = orders[m];
        const int64_t *a = A + offsets[m];
        if (n < 2 || !pg_exact_supported(a, n)) continue;
        double bits = 2.0;   // sign and rounding margin
        for (int i = 0; i < n; i++) {
            double b = 0;
            for (int j = 0; j < n; j++) b += std::fabs((double)a[(size_t)i * n + j]);
            bits += std::log2(std::max(1.0, b));
        }
        limbs = std::max(limbs, (int)std::ceil(bits / 32.0) + 1);
        exact_ids.push_back(m);
        poff.push_back((int64_t)packed.size());
        pord.push_back(n);
        packed.insert(packed.end(), a, a + (size_t)n * n);
    }
    std::vector<uint32_t> words((size_t)exact_ids.size() * limbs);
    if (!exact_ids.empty()) {
        const int st = pg_batch_exact(packed.data(), poff.data(), pord.data(),
                                      (int)exact_ids.size(), words.data(), limbs);
        if (st != PG_OK) return st;
    }
    std::vector<char> done(count, 0);
    for (size_t e = 0; e < exact_ids.size(); e++) {
        const int m = exact_ids[e];
        const uint32_t *w = words.data() + e * limbs;
        const bool negative = (w[limbs - 1] >> 31) != 0;
        for (int t = moduli_offsets[m]; t < moduli_offsets[m + 1]; t++) {
            const uint64_t p = moduli[t];
            // magnitude of the two's-complement value, Horner from the top limb
            uint64_t r = 0;
            uint32_t borrow = 1;
            std::vector<uint32_t> mag(w, w + limbs);
            if (negative) {
                for (int i = 0; i < limbs; i++) {   // -x = ~x + 1
                    const uint64_t v = (uint64_t)(uint32_t)~mag[i] + borrow;
                    mag[i] = (uint32_t)v;
                    borrow = (uint32_t)(v >> 32);
                }
            }
            for (int i = limbs - 1; i >= 0; i--)
                r = (uint64_t)((((unsigned __int128)r << 32) + mag[i]) % p);
            out[t] = negative && r ? p - r : r;
        }
        done[m] = 1;
    }
    for (int m = 0; m < count; m++) {
        if (done[m] || moduli_offsets[m + 1] == moduli_offsets[m]) continue;
        const int st = pg_residues(A + offsets[m], orders[m], moduli + moduli_offsets[m],
                                   moduli_offsets[m + 1] - moduli_offsets[m],
                                   out + moduli_offsets[m]);
        if (st != PG_OK) return st;
    }
    return PG_OK;
}

}  // extern "C"
