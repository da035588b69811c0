// Residue engine host logic and the wide-modulus kernels.
//
//  * odd m < 2^31   -> glynn_m32_kernel<N> (all such moduli in one launch)
//  * odd m < 2^32   -> glynn_m32_kernel<N, true> (fully reduced, 33-bit sums)
//  * odd m >= 2^32  -> glynn_m64_kernel (64-bit Montgomery, runtime n)
//  * even m = 2^e*o -> odd part as above, 2^e part from ryser_wrap64_kernel
//                      (Ryser in Z/2^64), recombined by CRT on the host
//
// Semantics follow rivin-perm perm_c_omp.c:846-854 / 858-929: entries are
// reduced mod m on the host (the C extension does this at :911), n < 64,
// per([]) = 1 mod m, per([[a]]) = a mod m.
#include "pg_internal.h"
#include "glynn_m32.cuh"

#include <vector>
#include <cstring>

namespace pg {

// ---------------------------------------------------------------------------
// 64-bit Montgomery Glynn (runtime n, row sums in local memory).  Used only
// for odd moduli >= 2^31; one thread per chunk, one partial per chunk.
__device__ __forceinline__ uint64_t m64_redc_mul(uint64_t a, uint64_t b,
                                                 uint64_t p, uint64_t pinv) {
    // a, b < p < 2^63: result in [0, p).
    const uint64_t lo = a * b, hi = __umul64hi(a, b);
    const uint64_t m = lo * pinv;
    uint64_t r = hi + __umul64hi(m, p) + (lo != 0);
    return r >= p ? r - p : r;
}
__device__ __forceinline__ uint64_t m64_add(uint64_t a, uint64_t b, uint64_t p) {
    return a >= p - b ? a - (p - b) : a + b;
}
__device__ __forceinline__ uint64_t m64_sub(uint64_t a, uint64_t b, uint64_t p) {
    return a >= b ? a - b : p - (b - a);
}

struct M64Args {
    const uint64_t *mats;     // [k][n*n] entries in [0, p)
    const uint64_t *moduli;   // [k]
    const uint64_t *pinvs;    // [k]
    uint64_t *partial;        // [k][chunks]
    int n;
    int log_len;
    uint64_t chunks;
    volatile const int *abort_flag;
    int *status;
};

__global__ void glynn_m64_kernel(M64Args a) {
    const int t = blockIdx.y;
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.chunks) return;
    if (*a.abort_flag) { atomicExch(a.status, 1); return; }
    const int n = a.n;
    const uint64_t p = a.moduli[t], pinv = a.pinvs[t];
    const uint64_t *m = a.mats + (size_t)t * n * n;
    uint64_t s[64];
    for (int i = 0; i < n; i++) {
        uint64_t v = 0;
        for (int j = 0; j < n; j++) v = m64_add(v, m[i * n + j], p);
        s[i] = v;
    }
    const uint64_t start = c << a.log_len, len = 1ull << a.log_len;
    const uint64_t g0 = start ^ (start >> 1);
    for (int j = 0; j < n - 1; j++)
        if ((g0 >> j) & 1)
            for (int i = 0; i < n; i++)
                s[i] = m64_sub(s[i], m64_add(m[i * n + j], m[i * n + j], p), p);
    int neg = __popcll(g0) & 1;
    uint64_t acc = 0;
    for (uint64_t i = 0; i < len; i++) {
        const uint64_t g = start + i;
        if (i) {
            const int j = __ffsll((long long)g) - 1;
            const int sub = ((g >> (j + 1)) & 1) == 0;
            for (int r = 0; r < n; r++) {
                const uint64_t d = m64_add(m[r * n + j], m[r * n + j], p);
                s[r] = sub ? m64_sub(s[r], d, p) : m64_add(s[r], d, p);
            }
            neg ^= 1;
        }
        uint64_t prod = s[0];
        for (int r = 1; r < n; r++) prod = m64_redc_mul(prod, s[r], p, pinv);
        acc = neg ? m64_sub(acc, prod, p) : m64_add(acc, prod, p);
    }
    a.partial[(size_t)t * a.chunks + c] = acc;
}

// Ryser over all 2^n subsets in Z/2^64 (entries taken as two's complement).
struct RyserArgs {
    const uint64_t *mat;   // n*n
    uint64_t *partial;     // [chunks]
    int n;
    int log_len;
    uint64_t chunks;
    volatile const int *abort_flag;
    int *status;
};

__global__ void ryser_wrap64_kernel(RyserArgs a) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.chunks) return;
    if (*a.abort_flag) { atomicExch(a.status, 1); return; }
    const int n = a.n;
    uint64_t s[64];
    for (int i = 0; i < n; i++) s[i] = 0;
    const uint64_t start = c << a.log_len, len = 1ull << a.log_len;
    const uint64_t g0 = start ^ (start >> 1);
    for (int j = 0; j < n; j++)
        if ((g0 >> j) & 1)
            for (int i = 0; i < n; i++) s[i] += a.mat[i * n + j];
    int neg = __popcll(g0) & 1;
    uint64_t acc = 0;
    for (uint64_t i = 0; i < len; i++) {
        const uint64_t g = start + i;
        if (i) {
            const int j = __ffsll((long long)g) - 1;
            const int add = (int)(((g ^ (g >> 1)) >> j) & 1);
            for (int r = 0; r < n; r++)
                s[r] = add ? s[r] + a.mat[r * n + j] : s[r] - a.mat[r * n + j];
            neg ^= 1;
        }
        uint64_t prod = s[0];
        for (int r = 1; r < n; r++) prod *= s[r];
        acc = neg ? acc - prod : acc + prod;
    }
    a.partial[c] = acc;
}

// ---------------------------------------------------------------------------
static cudaError_t launch_m32_any(int N, bool wide, const M32Args &args, int k, int bpm,
                                  cudaStream_t st) {
    if (wide) {
        if (N <= 22) return launch_glynn_m32w_lo(N, args, k, bpm, st);
        if (N <= 42) return launch_glynn_m32w_mid(N, args, k, bpm, st);
        return launch_glynn_m32w_hi(N, args, k, bpm, st);
    }
    if (N <= 22) return launch_glynn_m32_lo(N, args, k, bpm, st);
    if (N <= 42) return launch_glynn_m32_mid(N, args, k, bpm, st);
    return launch_glynn_m32_hi(N, args, k, bpm, st);
}
static int occupancy_m32_any(int N, bool wide) {
    if (wide) {
        if (N <= 22) return occupancy_glynn_m32w_lo(N);
        if (N <= 42) return occupancy_glynn_m32w_mid(N);
        return occupancy_glynn_m32w_hi(N);
    }
    if (N <= 22) return occupancy_glynn_m32_lo(N);
    if (N <= 42) return occupancy_glynn_m32_mid(N);
    return occupancy_glynn_m32_hi(N);
}

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// per(mats[t]) mod moduli[t] for odd moduli 3 <= m < 2^31, or for odd
// 2^31 <= m < 2^32 with `wide` (fully reduced form of the same kernel), n >= 2.
// With hi > 0, out[t] is instead the unscaled Glynn sum over Gray states
// [lo, hi) mod moduli[t] (no 2^(1-n) factor); lo and hi are multiples of 2.
static int glynn_m32_batch(const uint64_t *mats, int n, const uint64_t *moduli,
                           int k, bool wide, uint64_t *out, uint64_t lo = 0,
                           uint64_t hi = 0) {
    if (k > 65535) {   // grid.y limit: split into launches of <= 65535 moduli
        for (int t0 = 0; t0 < k; t0 += 65535) {
            const int kk = k - t0 < 65535 ? k - t0 : 65535;
            int st = glynn_m32_batch(mats + (size_t)t0 * n * n, n, moduli + t0, kk, wide,
                                     out + t0, lo, hi);
            if (st != PG_OK) return st;
        }
        return PG_OK;
    }
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;

    const int N = n, NCOL = n - 1, NP = (n + 3) & ~3;
    const size_t tab_words = (size_t)NCOL * 2 * NP;
    const size_t off_tab = 0;
    const size_t off_init = align_up(off_tab + (size_t)k * tab_words * 4, 256);
    const size_t off_mod = align_up(off_init + (size_t)k * NP * 4, 256);
    const size_t off_pinv = align_up(off_mod + (size_t)k * 4, 256);
    const size_t off_acc = align_up(off_pinv + (size_t)k * 4, 256);
    const size_t off_status = align_up(off_acc + (size_t)k * 8, 256);
    const size_t total = align_up(off_status + 16, 256);

    Workspace *ws;
    st = workspace(&ws, total, total);
    if (st != PG_OK) return st;
    char *h = (char *)ws->host;
    char *d = (char *)ws->dev;
    std::memset(h, 0, total);

    uint32_t *tab = (uint32_t *)(h + off_tab);
    uint32_t *init = (uint32_t *)(h + off_init);
    uint32_t *mods = (uint32_t *)(h + off_mod);
    uint32_t *pinvs = (uint32_t *)(h + off_pinv);
    for (int t = 0; t < k; t++) {
        const uint32_t p = (uint32_t)moduli[t];
        const uint64_t *m = mats + (size_t)t * n * n;
        mods[t] = p;
        pinvs[t] = neg_inv32(p);
        uint32_t *tt = tab + (size_t)t * tab_words;
        for (int j = 0; j < NCOL; j++) {
            for (int i = 0; i < N; i++) {
                const uint32_t two = (uint32_t)((2 * m[i * n + j]) % p);
                if (wide) {
                    tt[(2 * j + 0) * NP + i] = two;                // add
                    tt[(2 * j + 1) * NP + i] = two ? p - two : 0;  // sub
                } else {
                    tt[(2 * j + 0) * NP + i] = two - p;   // add: (s + two) mod p
                    tt[(2 * j + 1) * NP + i] = 0u - two;  // sub: (s - two) mod p
                }
            }
        }
        for (int i = 0; i < N; i++) {
            uint64_t v = 0;
            for (int j = 0; j < n; j++) v += m[i * n + j];
            init[(size_t)t * NP + i] = (uint32_t)(v % p);
        }
    }

    // Launch shape: one resident wave of blocks shared by the k moduli; each
    // thread owns a contiguous range of ~128 chunks of >= 64 states (small
    // orders use fewer blocks so every thread keeps >= 512 states).
    const int occ = occupancy_m32_any(N, wide);
    const int log_states = n - 1;
    const bool partial = hi > 0;
    const uint64_t span = partial ? hi - lo : 1ull << log_states;
    uint64_t bpm = ((uint64_t)occ * dev.sm_count + k - 1) / k;
    while (bpm > 1 && (span >> 9) < bpm * 256) bpm >>= 1;
    if (bpm < 1) bpm = 1;
    if (bpm > 65535) bpm = 65535;
    int log_T = 0;
    while ((2ull << log_T) <= bpm * 256) log_T++;
    ChunkPlan pl;
    pl.log_len = log_states - (log_T + 7);
    const int min_len = log_states < 6 ? log_states : 6;
    if (pl.log_len < min_len) pl.log_len = min_len;
    if (pl.log_len > 30) pl.log_len = 30;
    if (pl.log_len < 1) pl.log_len = 1;
    pl.chunks = 1ull << (log_states - pl.log_len);

    uint64_t chunk0 = 0;
    if (partial) {
        // about 128 chunks per thread over the window, shortened until the
        // chunk length divides lo and hi; the kernel steps 2 states per
        // iteration
        int log_span = 0;
        while ((2ull << log_span) <= span) log_span++;
        int ll = log_span - (log_T + 7);
        if (ll > 30) ll = 30;
        if (ll < 1) ll = 1;
        while (ll > 1 && ((lo | hi) & ((1ull << ll) - 1))) ll--;
        pl.log_len = ll;
        pl.chunks = span >> ll;
        chunk0 = lo >> ll;
    }
    M32Args args;
    args.tabs = (const uint32_t *)(d + off_tab);
    args.init = (const uint32_t *)(d + off_init);
    args.moduli = (const uint32_t *)(d + off_mod);
    args.pinvs = (const uint32_t *)(d + off_pinv);
    args.acc = (unsigned long long *)(d + off_acc);
    args.status = (int *)(d + off_status);
    args.abort_flag = abort_dev;
    args.chunks = pl.chunks;
    args.log_len = pl.log_len;
    args.chunk0 = chunk0;

    PG_CUDA(cudaMemcpyAsync(d, h, off_acc, cudaMemcpyHostToDevice, ws->stream));
    PG_CUDA(cudaMemsetAsync(d + off_acc, 0, total - off_acc, ws->stream));
    PG_CUDA(launch_m32_any(N, wide, args, k, (int)bpm, ws->stream));
    PG_CUDA(cudaMemcpyAsync(h + off_acc, d + off_acc, total - off_acc,
                            cudaMemcpyDeviceToHost, ws->stream));
    PG_CUDA(cudaStreamSynchronize(ws->stream));
    if (*(int *)(h + off_status))
        return fail(PG_EABORT, "residue launch aborted by pg_abort()");

    const unsigned long long *acc = (const unsigned long long *)(h + off_acc);
    for (int t = 0; t < k; t++) {
        const uint64_t p = moduli[t];
        const uint64_t R = (1ull << 32) % p;
        const uint64_t inv2 = (p >> 1) + 1;
        uint64_t r = acc[t] % p;
        r = mulmod_u64(r, powmod_u64(R, (uint64_t)(n - 1), p), p);
        if (!partial) r = mulmod_u64(r, powmod_u64(inv2, (uint64_t)(n - 1), p), p);
        out[t] = r;
    }
    return PG_OK;
}

// per(mats[t]) mod moduli[t] for odd moduli >= 2^31 (< 2^63), n >= 2.
static int glynn_m64_batch(const uint64_t *mats, int n, const uint64_t *moduli,
                           int k, uint64_t *out) {
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    ChunkPlan pl = plan_chunks(n - 1, 0, (uint64_t)dev.sm_count * 512);
    const size_t nn = (size_t)n * n;
    const size_t off_mat = 0;
    const size_t off_mod = align_up(off_mat + k * nn * 8, 256);
    const size_t off_pinv = align_up(off_mod + (size_t)k * 8, 256);
    const size_t off_status = align_up(off_pinv + (size_t)k * 8, 256);
    const size_t off_part = align_up(off_status + 16, 256);
    const size_t total = align_up(off_part + (size_t)k * pl.chunks * 8, 256);
    Workspace *ws;
    st = workspace(&ws, total, total);
    if (st != PG_OK) return st;
    char *h = (char *)ws->host;
    char *d = (char *)ws->dev;
    std::memcpy(h + off_mat, mats, k * nn * 8);
    for (int t = 0; t < k; t++) {
        ((uint64_t *)(h + off_mod))[t] = moduli[t];
        ((uint64_t *)(h + off_pinv))[t] = neg_inv64(moduli[t]);
    }
    *(int *)(h + off_status) = 0;
    M64Args a;
    a.mats = (const uint64_t *)(d + off_mat);
    a.moduli = (const uint64_t *)(d + off_mod);
    a.pinvs = (const uint64_t *)(d + off_pinv);
    a.partial = (uint64_t *)(d + off_part);
    a.n = n;
    a.log_len = pl.log_len;
    a.chunks = pl.chunks;
    a.abort_flag = abort_dev;
    a.status = (int *)(d + off_status);
    PG_CUDA(cudaMemcpyAsync(d, h, off_part, cudaMemcpyHostToDevice, ws->stream));
    dim3 grid((unsigned)((pl.chunks + 127) / 128), (unsigned)k);
    glynn_m64_kernel<<<grid, 128, 0, ws->stream>>>(a);
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaMemcpyAsync(h + off_status, d + off_status, total - off_status,
                            cudaMemcpyDeviceToHost, ws->stream));
    PG_CUDA(cudaStreamSynchronize(ws->stream));
    if (*(int *)(h + off_status))
        return fail(PG_EABORT, "residue launch aborted by pg_abort()");
    const uint64_t *part = (const uint64_t *)(h + off_part);
    for (int t = 0; t < k; t++) {
        const uint64_t p = moduli[t];
        uint64_t r = 0;
        for (uint64_t c = 0; c < pl.chunks; c++) {
            r += part[(size_t)t * pl.chunks + c];
            if (r >= p) r -= p;
        }
        const uint64_t R = (uint64_t)(((unsigned __int128)1 << 64) % p);
        r = mulmod_u64(r, powmod_u64(R, (uint64_t)(n - 1), p), p);
        r = mulmod_u64(r, powmod_u64((p >> 1) + 1, (uint64_t)(n - 1), p), p);
        out[t] = r;
    }
    return PG_OK;
}

int glynn_residues_odd(const uint64_t *mats, int n, const uint64_t *moduli,
                       int k, uint64_t *out) {
    // n >= 2, every modulus odd and >= 3: m < 2^31 narrow 32-bit kernel,
    // m < 2^32 its wide form, larger moduli the 64-bit kernel
    std::vector<int> cls[3];
    for (int t = 0; t < k; t++)
        cls[moduli[t] < (1ull << 31) ? 0 : moduli[t] < (1ull << 32) ? 1 : 2].push_back(t);
    const size_t nn = (size_t)n * n;
    for (int pass = 0; pass < 3; pass++) {
        const std::vector<int> &idx = cls[pass];
        if (idx.empty()) continue;
        std::vector<uint64_t> m(idx.size() * nn), mod(idx.size()), res(idx.size());
        for (size_t q = 0; q < idx.size(); q++) {
            std::memcpy(&m[q * nn], mats + idx[q] * nn, nn * 8);
            mod[q] = moduli[idx[q]];
        }
        int st = pass < 2
                     ? glynn_m32_batch(m.data(), n, mod.data(), (int)idx.size(), pass == 1,
                                       res.data())
                     : glynn_m64_batch(m.data(), n, mod.data(), (int)idx.size(), res.data());
        if (st != PG_OK) return st;
        for (size_t q = 0; q < idx.size(); q++) out[idx[q]] = res[q];
    }
    return PG_OK;
}

int ryser_wrap64(const int64_t *A, int n, uint64_t *out) {
    // per(A) mod 2^64 for n >= 1.
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    ChunkPlan pl = plan_chunks(n, 0, (uint64_t)dev.sm_count * 512);
    const size_t nn = (size_t)n * n;
    const size_t off_status = align_up(nn * 8, 256);
    const size_t off_part = align_up(off_status + 16, 256);
    const size_t total = align_up(off_part + pl.chunks * 8, 256);
    Workspace *ws;
    st = workspace(&ws, total, total);
    if (st != PG_OK) return st;
    char *h = (char *)ws->host;
    char *d = (char *)ws->dev;
    std::memcpy(h, A, nn * 8);
    *(int *)(h + off_status) = 0;
    RyserArgs a;
    a.mat = (const uint64_t *)d;
    a.partial = (uint64_t *)(d + off_part);
    a.n = n;
    a.log_len = pl.log_len;
    a.chunks = pl.chunks;
    a.abort_flag = abort_dev;
    a.status = (int *)(d + off_status);
    PG_CUDA(cudaMemcpyAsync(d, h, off_part, cudaMemcpyHostToDevice, ws->stream));
    ryser_wrap64_kernel<<<(unsigned)((pl.chunks + 127) / 128), 128, 0, ws->stream>>>(a);
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaMemcpyAsync(h + off_status, d + off_status, total - off_status,
                            cudaMemcpyDeviceToHost, ws->stream));
    PG_CUDA(cudaStreamSynchronize(ws->stream));
    if (*(int *)(h + off_status))
        return fail(PG_EABORT, "residue launch aborted by pg_abort()");
    uint64_t r = 0;
    const uint64_t *part = (const uint64_t *)(h + off_part);
    for (uint64_t c = 0; c < pl.chunks; c++) r += part[c];
    if (n & 1) r = 0 - r;
    *out = r;
    return PG_OK;
}

// Full residue contract for one integer matrix and k arbitrary moduli.
static int residues_impl(const int64_t *A, int n, const uint64_t *moduli, int k,
                         uint64_t *out) {
    if (n == 0) {
        for (int t = 0; t < k; t++) out[t] = 1 % moduli[t];
        return PG_OK;
    }
    if (n == 1) {
        for (int t = 0; t < k; t++) out[t] = normmod_i64(A[0], moduli[t]);
        return PG_OK;
    }
    const size_t nn = (size_t)n * n;
    std::vector<uint64_t> odd_mod, odd_res, mats;
    std::vector<int> odd_of(k, -1);
    bool need_two = false;
    for (int t = 0; t < k; t++) {
        const uint64_t m = moduli[t];
        if (m == 1) continue;
        const int e = __builtin_ctzll(m);
        const uint64_t o = m >> e;
        if (e) need_two = true;
        if (o > 1) {
            odd_of[t] = (int)odd_mod.size();
            odd_mod.push_back(o);
        }
    }
    if (!odd_mod.empty()) {
        mats.resize(odd_mod.size() * nn);
        for (size_t q = 0; q < odd_mod.size(); q++)
            for (size_t i = 0; i < nn; i++) mats[q * nn + i] = normmod_i64(A[i], odd_mod[q]);
        odd_res.resize(odd_mod.size());
        int st = glynn_residues_odd(mats.data(), n, odd_mod.data(),
                                    (int)odd_mod.size(), odd_res.data());
        if (st != PG_OK) return st;
    }
    uint64_t two_res = 0;
    if (need_two) {
        int st = ryser_wrap64(A, n, &two_res);
        if (st != PG_OK) return st;
    }
    for (int t = 0; t < k; t++) {
        const uint64_t m = moduli[t];
        if (m == 1) { out[t] = 0; continue; }
        const int e = __builtin_ctzll(m);
        const uint64_t o = m >> e;
        if (e == 0) { out[t] = odd_res[odd_of[t]]; continue; }
        const uint64_t mask = e >= 64 ? ~0ull : ((1ull << e) - 1);
        const uint64_t r2 = two_res & mask;
        if (o == 1) { out[t] = r2; continue; }
        // x = ro + o * ((r2 - ro) * o^-1 mod 2^e)
        const uint64_t ro = odd_res[odd_of[t]];
        uint64_t inv = o;
        for (int i = 0; i < 6; i++) inv *= 2 - o * inv;  // o^-1 mod 2^64
        const uint64_t tq = ((r2 - ro) * inv) & mask;
        out[t] = (uint64_t)((ro + (unsigned __int128)o * tq) % m);
    }
    return PG_OK;
}

static int check_moduli(const uint64_t *moduli, int k) {
    if (k < 0) return fail(PG_EINVAL, "k must be non-negative");
    if (k > 0 && !moduli) return fail(PG_EINVAL, "moduli is null");
    for (int t = 0; t < k; t++)
        if (moduli[t] == 0 || moduli[t] >= (1ull << 63))
            return fail(PG_ERANGE, "moduli must satisfy 1 <= m < 2^63");
    return PG_OK;
}

static bool is_prime_u64(uint64_t v) {
    static const uint64_t small[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (v < 2) return false;
    for (uint64_t p : small) {
        if (v == p) return true;
        if (v % p == 0) return false;
    }
    uint64_t d = v - 1;
    int r = 0;
    while (!(d & 1)) { d >>= 1; r++; }
    static const uint64_t wit[] = {2, 325, 9375, 28178, 450775, 9780504, 1795265022};
    for (uint64_t b : wit) {
        b %= v;
        if (!b) continue;
        uint64_t x = powmod_u64(b, d, v);
        if (x == 1 || x == v - 1) continue;
        bool comp = true;
        for (int i = 1; i < r; i++) {
            x = mulmod_u64(x, x, v);
            if (x == v - 1) { comp = false; break; }
        }
        if (comp) return false;
    }
    return true;
}

}  // namespace pg

extern "C" {

int pg_residues(const int64_t *A, int n, const uint64_t *moduli, int k,
                uint64_t *out) {
    using namespace pg;
    if (n < 0 || n >= 64) return fail(PG_ERANGE, "matrix dimension must be less than 64");
    if (n > 0 && !A) return fail(PG_EINVAL, "matrix is null");
    if (k > 0 && !out) return fail(PG_EINVAL, "out is null");
    int st = check_moduli(moduli, k);
    if (st != PG_OK) return st;
    if (k == 0) return PG_OK;
    return residues_impl(A, n, moduli, k, out);
}

int pg_residues_partial(const int64_t *A, int n, uint64_t state_lo, uint64_t state_hi,
                        const uint64_t *moduli, int k, uint64_t *out) {
    using namespace pg;
    if (n < 2 || n >= 64) return fail(PG_ERANGE, "partial residues need 2 <= n < 64");
    if (!A) return fail(PG_EINVAL, "matrix is null");
    if (k > 0 && (!moduli || !out)) return fail(PG_EINVAL, "null argument");
    const uint64_t states = 1ull << (n - 1);
    if (state_lo >= state_hi || state_hi > states)
        return fail(PG_ERANGE, "state range must satisfy lo < hi <= 2^(n-1)");
    if ((state_lo | state_hi) & 1) return fail(PG_EINVAL, "state range bounds must be even");
    for (int t = 0; t < k; t++)
        if (moduli[t] < 3 || !(moduli[t] & 1) || moduli[t] >= (1ull << 32))
            return fail(PG_ERANGE, "partial residues need odd moduli 3 <= m < 2^32");
    const size_t nn = (size_t)n * n;
    for (int wide = 0; wide < 2; wide++) {
        std::vector<uint64_t> mats, mods;
        std::vector<int> idx;
        for (int t = 0; t < k; t++) {
            if ((moduli[t] >= (1ull << 31)) != (wide == 1)) continue;
            const size_t base = mats.size();
            mats.resize(base + nn);
            for (size_t i = 0; i < nn; i++) mats[base + i] = normmod_i64(A[i], moduli[t]);
            mods.push_back(moduli[t]);
            idx.push_back(t);
        }
        if (idx.empty()) continue;
        std::vector<uint64_t> res(idx.size());
        const int st = glynn_m32_batch(mats.data(), n, mods.data(), (int)idx.size(), wide == 1,
                                       res.data(), state_lo, state_hi);
        if (st != PG_OK) return st;
        for (size_t q = 0; q < idx.size(); q++) out[idx[q]] = res[q];
    }
    return PG_OK;
}

int pg_schur_residues(int n, const uint64_t *primes, const uint64_t *omegas,
                      int k, uint64_t *out) {
    return pg_schur_residues_method(n, primes, omegas, k, PG_SCHUR_AUTO, out);
}

int pg_schur_residues_method(int n, const uint64_t *primes, const uint64_t *omegas,
                             int k, int method, uint64_t *out) {
    using namespace pg;
    if (n < 0 || n >= 64) return fail(PG_ERANGE, "n must satisfy 0 <= n < 64");
    if (k > 0 && (!omegas || !out)) return fail(PG_EINVAL, "null argument");
    if (method != PG_SCHUR_AUTO && method != PG_SCHUR_GLYNN && method != PG_SCHUR_NECKLACE)
        return fail(PG_EINVAL, "unknown Schur method");
    int st = check_moduli(primes, k);
    if (st != PG_OK) return st;
    std::vector<uint64_t> minor_mod, minor_mats;
    std::vector<int> minor_of(k, -1);
    std::vector<uint64_t> neck_p, neck_w;
    std::vector<int> neck_of;
    for (int t = 0; t < k; t++) {
        const uint64_t p = primes[t];
        if (n <= 1) { out[t] = 1 % p; continue; }
        if (p == 1) { out[t] = 0; continue; }
        const uint64_t w = omegas[t] % p;
        const bool cofactor =
            n >= 3 && (n & 1) && (p & 1) && powmod_u64(w, (uint64_t)n, p) == 1 % p;
        const bool necklace =
            cofactor && necklace_supported(n) &&
            (p < NECKLACE_PRIME_LIMIT ||
             (p < NECKLACE_WIDE_PRIME_LIMIT && necklace_wide_supported(n)));
        if (method == PG_SCHUR_NECKLACE && !necklace)
            return fail(PG_ERANGE, "necklace quotient needs an odd prime n < 64, an odd "
                                   "modulus below 2^30 (2^32 for n >= 37) and omega^n == 1");
        if (necklace && (method == PG_SCHUR_NECKLACE ||
                         (method == PG_SCHUR_AUTO && n >= NECKLACE_AUTO_MIN_ORDER))) {
            neck_of.push_back(t);
            neck_p.push_back(p);
            neck_w.push_back(w);
        } else if (cofactor) {
            // n * per(minor), minor[r][c] = w^((r+1)(c+1)), (n-1) x (n-1)
            const int q = n - 1;
            minor_of[t] = (int)minor_mod.size();
            minor_mod.push_back(p);
            size_t base = minor_mats.size();
            minor_mats.resize(base + (size_t)q * q);
            uint64_t wj = w;
            for (int r = 0; r < q; r++) {
                uint64_t pw = wj;
                for (int c = 0; c < q; c++) {
                    minor_mats[base + (size_t)r * q + c] = pw;
                    pw = mulmod_u64(pw, wj, p);
                }
                wj = mulmod_u64(wj, w, p);
            }
        } else {
            // full matrix S[j][c] = w^(j c) mod p through the generic path
            std::vector<int64_t> full((size_t)n * n);
            uint64_t wj = 1 % p;
            for (int r = 0; r < n; r++) {
                uint64_t pw = 1 % p;
                for (int c = 0; c < n; c++) {
                    full[(size_t)r * n + c] = (int64_t)pw;
                    pw = mulmod_u64(pw, wj, p);
                }
                wj = mulmod_u64(wj, w, p);
            }
            st = residues_impl(full.data(), n, &primes[t], 1, &out[t]);
            if (st != PG_OK) return st;
        }
    }
    if (!minor_mod.empty()) {
        std::vector<uint64_t> res(minor_mod.size());
        st = glynn_residues_odd(minor_mats.data(), n - 1, minor_mod.data(),
                                (int)minor_mod.size(), res.data());
        if (st != PG_OK) return st;
        for (int t = 0; t < k; t++)
            if (minor_of[t] >= 0)
                out[t] = mulmod_u64(res[minor_of[t]], (uint64_t)n % primes[t], primes[t]);
    }
    if (!neck_p.empty()) {
        std::vector<uint64_t> res(neck_p.size());
        st = schur_necklace_residues(n, neck_p.data(), neck_w.data(), (int)neck_p.size(),
                                     res.data());
        if (st != PG_OK) return st;
        for (size_t i = 0; i < neck_of.size(); i++) out[neck_of[i]] = res[i];
    }
    return PG_OK;
}

int pg_binary_residues(const uint8_t *A, int n, const uint64_t *primes, int k,
                       uint64_t *out) {
    using namespace pg;
    if (n < 0 || n >= 64) return fail(PG_ERANGE, "native binary backend supports order at most 63");
    if (n > 0 && !A) return fail(PG_EINVAL, "matrix is null");
    if (k > 0 && (!primes || !out)) return fail(PG_EINVAL, "null argument");
    if (k < 0) return fail(PG_EINVAL, "k must be non-negative");
    for (int t = 0; t < k; t++) {
        const uint64_t p = primes[t];
        if (p <= 1 || p >= (1ull << 63)) return fail(PG_ERANGE, "p must be greater than 1");
        if (p == 2) return fail(PG_ERANGE, "p must be odd");
        if (p <= (uint64_t)n) return fail(PG_ERANGE, "p must be greater than the matrix order");
        if (!is_prime_u64(p)) return fail(PG_ERANGE, "p must be prime");
    }
    const size_t nn = (size_t)n * n;
    for (size_t i = 0; i < nn; i++)
        if (A[i] > 1) return fail(PG_EINVAL, "binary matrix entries must be 0 or 1");
    if (k == 0) return PG_OK;
    if (n <= 1) {
        for (int t = 0; t < k; t++) out[t] = n == 0 ? 1 % primes[t] : A[0] % primes[t];
        return PG_OK;
    }
    std::vector<uint64_t> mats((size_t)k * nn);
    for (int t = 0; t < k; t++)
        for (size_t i = 0; i < nn; i++) mats[(size_t)t * nn + i] = A[i];
    return glynn_residues_odd(mats.data(), n, primes, k, out);
}

}  // extern "C"
