// Necklace quotient for Schur permanents of prime order n.
//
// For prime n the (n-1)x(n-1) cofactor minor w^((r+1)(c+1)) becomes
// circulant after indexing rows and columns by powers of a primitive root
// g (mod n): M[r][c] = f[(c - r) mod L], f[k] = w^(g^k mod n), L = n - 1
// (rivin-perm perm_c_omp.c:193-214).  The Glynn term of a sign word over all
// 2^L words is invariant under cyclic rotation of the word and, L being
// even, under complement, so
//   per(M) = 2^-L sum_{orbit representatives w} |orbit(w)| (-1)^|w| prod_i s_i(w)
// with representatives = binary necklaces of weight <= L/2 (a weight-L/2
// necklace is kept only if it is not larger than the least rotation of its
// complement) and |orbit| = 2 * period, or period for a self-complementary
// orbit (perm_c_omp.c:81-121, 249-284).  About 2^L / (2L) terms instead of
// the 2^(L-1) Glynn states of the minor.
//
// GPU organisation: the host enumerates FKM subtree roots (prefixes of a
// fixed depth, packed into 32-bit words); every thread takes roots from a
// per-prime atomic counter and walks its subtree with the iterative FKM
// successor on one 64-bit word (rightmost free 0 becomes 1, then periodic
// extension by doubling), skipping every subtree whose prefix weight already
// exceeds L/2.  Row sums mod p are updated only at the bits that changed
// since the last evaluated word, from a per-column table in shared memory,
// and each accepted term is formed with the Montgomery chain of the Glynn
// residue kernel.  All primes run in one launch (grid.y = prime).  The
// walker is __host__ __device__: pg_necklace_orbit_stats counts
// representatives and covered words with the very same code on the host.
#include "pg_internal.h"
#include "glynn_m32.cuh"

#include <cstring>
#include <vector>

namespace pg {

// Root word: prefix bits a[1..depth] (a[1] most significant) in bits 0..25,
// Lyndon period of the prefix in bits 26..31.
constexpr int NK_MAX_DEPTH = 26;

__host__ __device__ __forceinline__ int nk_popc(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}
__host__ __device__ __forceinline__ int nk_ctz(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __ffsll((long long)x) - 1;
#else
    return __builtin_ctzll(x);
#endif
}

// L-bit word whose first m bits (the top m bits) are `pat` and whose later
// bits repeat with period m.
__host__ __device__ __forceinline__ uint64_t nk_extend(uint64_t pat, int m, int L) {
    uint64_t cur = pat;
    int len = m;
    while (2 * len <= L) {
        cur = (cur << len) | cur;
        len *= 2;
    }
    if (len == L) return cur;
    return (cur << (L - len)) | (cur >> (2 * len - L));
}

__host__ __device__ __forceinline__ uint64_t nk_least_rotation(uint64_t w, int L) {
    const uint64_t mask = (1ull << L) - 1;
    uint64_t best = w;
    for (int s = 1; s < L; s++) {
        const uint64_t r = ((w << s) | (w >> (L - s))) & mask;
        best = r < best ? r : best;
    }
    return best;
}

// Orbit size of necklace w (period p) when w is the chosen representative
// of its rotation+complement orbit, else 0.
__host__ __device__ __forceinline__ uint32_t nk_orbit(uint64_t w, int p, int L) {
    const int weight = nk_popc(w), half = L / 2;
    if (weight < half) return 2u * p;
    if (weight > half) return 0;
    const uint64_t cr = nk_least_rotation(~w & ((1ull << L) - 1), L);
    if (w > cr) return 0;
    return w == cr ? (uint32_t)p : 2u * p;
}

// Walk the FKM subtree of `root` (lexicographic order of pre-necklaces
// sharing the root's prefix), calling visit(word, orbit) for every accepted
// representative.
template <class Visit>
__host__ __device__ __forceinline__ void nk_walk(uint32_t root, int depth, int L,
                                                Visit &visit) {
    const int half = L / 2;
    int p = (int)(root >> NK_MAX_DEPTH);
    const uint64_t prefix = root & ((1u << NK_MAX_DEPTH) - 1);
    uint64_t w = nk_extend(prefix >> (depth - p), p, L);
    const uint64_t free_mask = (1ull << (L - depth)) - 1;
    bool emit = true;
    for (;;) {
        if (emit && L % p == 0) {
            const uint32_t orb = nk_orbit(w, p, L);
            if (orb) visit(w, orb);
        }
        const uint64_t free = ~w & free_mask;
        if (!free) break;
        const int b = nk_ctz(free);          // rightmost 0: position i = L - b
        const uint64_t pre = (w >> b) | 1ull;
        if (nk_popc(pre) > half) {
            // every word below this prefix is heavier than L/2: fill the
            // tail with ones so the next successor moves left of it
            w = (pre << b) | ((1ull << b) - 1);
            emit = false;
            continue;
        }
        p = L - b;
        w = nk_extend(pre, p, L);
        emit = true;
    }
}

// Host: FKM subtree roots at prefix depth `depth`, prefix weight <= L/2
// (perm_c_omp.c:375-402 collects subtree states the same way for its
// CPU threads).
static void nk_roots_rec(std::vector<uint32_t> &out, uint8_t *a, int t, int period,
                         int weight, uint32_t prefix, int L, int depth) {
    if (t > depth) {
        out.push_back(prefix | ((uint32_t)period << NK_MAX_DEPTH));
        return;
    }
    const uint8_t bit = a[t - period];
    if (weight + bit <= L / 2) {
        a[t] = bit;
        nk_roots_rec(out, a, t + 1, period, weight + bit, (prefix << 1) | bit, L, depth);
    }
    if (bit == 0 && weight + 1 <= L / 2) {
        a[t] = 1;
        nk_roots_rec(out, a, t + 1, t, weight + 1, (prefix << 1) | 1u, L, depth);
    }
}

static std::vector<uint32_t> nk_roots(int L, int depth) {
    std::vector<uint32_t> out;
    uint8_t a[NK_MAX_DEPTH + 2] = {0};
    nk_roots_rec(out, a, 1, 1, 0, 0, L, depth);
    return out;
}

// Subtrees of at most 2^14 words keep the largest work item well below a
// thread's share; 26 bits bound the root table (a few million roots).
static int nk_depth(int L) {
    int d = L - 14;
    if (d > NK_MAX_DEPTH) d = NK_MAX_DEPTH;
    if (d < 1) d = 1;
    return d;
}

// Table row stride in words: a multiple of 4 with an odd count of 16-byte
// units, so 128-bit reads of different columns spread over the banks.
__host__ __device__ constexpr int nk_stride(int L) {
    return ((L + 3) / 4 % 2 == 1) ? (L + 3) / 4 * 4 : (L + 3) / 4 * 4 + 4;
}

struct NeckArgs {
    const uint32_t *tabs;     // [k][L][2][LS] (d - p) mod 2^32; 0 bit clear, 1 set
    const uint32_t *init;     // [k] row sum of the all-plus word (equal for all rows)
    const uint32_t *moduli;
    const uint32_t *pinvs;
    const uint32_t *roots;
    uint32_t nroots;
    int depth;
    unsigned int *counters;   // [k] root counters (zeroed)
    unsigned long long *acc;  // [k] (zeroed)
    volatile const int *abort_flag;
    int *status;
};

template <int L>
struct NeckEval {
    static constexpr int LS = nk_stride(L);
    uint32_t s[L];
    uint64_t prev;
    const uint32_t *tab;
    uint32_t p, pinv;
    unsigned long long pos, neg;
    uint32_t count;

    __device__ __forceinline__ void add_column(const uint32_t *c) {
        const uint4 *c4 = reinterpret_cast<const uint4 *>(c);
#pragma unroll
        for (int q = 0; q < L / 4; q++) {
            const uint4 v = c4[q];
            s[4 * q + 0] = m32_addmod(s[4 * q + 0], v.x, p);
            s[4 * q + 1] = m32_addmod(s[4 * q + 1], v.y, p);
            s[4 * q + 2] = m32_addmod(s[4 * q + 2], v.z, p);
            s[4 * q + 3] = m32_addmod(s[4 * q + 3], v.w, p);
        }
        if constexpr (L % 4 != 0) {
            const uint2 v = reinterpret_cast<const uint2 *>(c)[(L - 2) / 2];
            s[L - 2] = m32_addmod(s[L - 2], v.x, p);
            s[L - 1] = m32_addmod(s[L - 1], v.y, p);
        }
    }

    __device__ __forceinline__ void operator()(uint64_t w, uint32_t orbit) {
        uint64_t diff = w ^ prev;
        prev = w;
        while (diff) {
            const int bit = nk_ctz(diff);
            diff &= diff - 1;
            const int col = L - 1 - bit;
            const int set = (int)((w >> bit) & 1);
            add_column(tab + (2 * col + set) * LS);
        }
        uint32_t prod;
        if constexpr (L < 4) {
            prod = s[0];
#pragma unroll
            for (int i = 1; i < L; i++) prod = m32_redc_mul(prod, s[i], p, pinv);
        } else {
            uint32_t ch[4] = {s[0], s[1], s[2], s[3]};
#pragma unroll
            for (int i = 4; i < L; i++) ch[i & 3] = m32_redc_mul(ch[i & 3], s[i], p, pinv);
            const uint32_t c1 = __viaddmin_u32(ch[1], 0u - p, ch[1]);
            const uint32_t c3 = __viaddmin_u32(ch[3], 0u - p, ch[3]);
            const uint32_t c01 = m32_redc_mul(ch[0], c1, p, pinv);
            const uint32_t c23 = m32_redc_mul(ch[2], c3, p, pinv);
            prod = m32_redc_mul(c01, __viaddmin_u32(c23, 0u - p, c23), p, pinv);
        }
        const unsigned long long t = (unsigned long long)prod * orbit;
        if (nk_popc(w) & 1) neg += t;
        else pos += t;
        if (++count == (1u << 20)) {     // prod*orbit < 2^39: reduce long before 2^64
            pos %= p;
            neg %= p;
            count = 0;
        }
    }
};

template <int L>
__global__ void __launch_bounds__(256) necklace_m32_kernel(NeckArgs a) {
    constexpr int LS = nk_stride(L);
    extern __shared__ uint4 nsm[];
    const int k = blockIdx.y;
    {
        const uint4 *g = reinterpret_cast<const uint4 *>(a.tabs + (size_t)k * L * 2 * LS);
        for (int i = threadIdx.x; i < L * 2 * LS / 4; i += blockDim.x) nsm[i] = g[i];
    }
    __syncthreads();
    NeckEval<L> ev;
    ev.tab = reinterpret_cast<const uint32_t *>(nsm);
    ev.p = a.moduli[k];
    ev.pinv = a.pinvs[k];
    ev.pos = ev.neg = 0;
    ev.count = 0;
    const uint32_t s0 = a.init[k];
    bool aborted = false;
    for (;;) {
        const unsigned int r = atomicAdd(a.counters + k, 1u);
        if (r >= a.nroots) break;
        if (*a.abort_flag) {
            aborted = true;
            break;
        }
        // start from the all-plus word: the first evaluation applies every
        // set bit of the subtree's first word as a change
#pragma unroll
        for (int i = 0; i < L; i++) ev.s[i] = s0;
        ev.prev = 0;
        nk_walk(a.roots[r], a.depth, L, ev);
    }
    const uint32_t p = ev.p;
    unsigned long long v = ev.pos % p + (p - ev.neg % p);
    v %= p;
    __shared__ unsigned long long red[8];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < 8; w++) t += red[w];
        atomicAdd(a.acc + k, t);
    }
    if (aborted) atomicExch(a.status, 1);
}

// Minor orders L = n - 1 of the odd primes 3 .. 61.
#define PG_NK_ORDERS(X) X(2) X(4) X(6) X(10) X(12) X(16) X(18) X(22) X(28) X(30) \
                        X(36) X(40) X(42) X(46) X(52) X(58) X(60)

bool necklace_supported(int n) {
    switch (n - 1) {
#define PG_NK_YES(LL) case LL:
        PG_NK_ORDERS(PG_NK_YES)
#undef PG_NK_YES
        return true;
    default:
        return false;
    }
}

static cudaError_t launch_necklace(int L, const NeckArgs &a, int k, int sm_count,
                                   cudaStream_t s) {
    const size_t smem = (size_t)L * 2 * nk_stride(L) * 4;
    switch (L) {
#define PG_NK_CASE(LL)                                                                    \
    case LL: {                                                                            \
        cudaError_t e = cudaFuncSetAttribute(necklace_m32_kernel<LL>,                     \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                             (int)smem);                                  \
        if (e != cudaSuccess) return e;                                                   \
        int per_sm = 0;                                                                   \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, necklace_m32_kernel<LL>, \
                                                          256, smem);                     \
        if (e != cudaSuccess) return e;                                                   \
        if (per_sm < 1) per_sm = 1;                                                       \
        int bpm = (per_sm * sm_count + k - 1) / k;                                        \
        dim3 grid(bpm, k);                                                                \
        necklace_m32_kernel<LL><<<grid, 256, smem, s>>>(a);                               \
        return cudaGetLastError();                                                        \
    }
        PG_NK_ORDERS(PG_NK_CASE)
#undef PG_NK_CASE
    default:
        return cudaErrorInvalidValue;
    }
}

static size_t nk_align(size_t v) { return (v + 255) / 256 * 256; }

static int primitive_root_of_prime(int q) {
    const int phi = q - 1;
    int f[16], nf = 0, r = phi;
    for (int d = 2; d * d <= r; d++)
        if (r % d == 0) {
            f[nf++] = d;
            while (r % d == 0) r /= d;
        }
    if (r > 1) f[nf++] = r;
    for (int g = 2; g < q; g++) {
        bool ok = true;
        for (int t = 0; t < nf && ok; t++)
            if (powmod_u64((uint64_t)g, (uint64_t)(phi / f[t]), (uint64_t)q) == 1) ok = false;
        if (ok) return g;
    }
    return -1;
}

// n * per(circulant Schur minor) mod primes[t] = perm(S_n) mod primes[t],
// for prime n with necklace_supported(n), odd primes[t] < 2^31 and
// omegas[t]^n == 1 (mod primes[t]).
int schur_necklace_residues(int n, const uint64_t *primes, const uint64_t *omegas, int k,
                            uint64_t *out) {
    if (k <= 0) return PG_OK;
    const int L = n - 1, LS = nk_stride(L);
    const int g = primitive_root_of_prime(n);
    if (g < 0 || !necklace_supported(n)) return fail(PG_EINTERNAL, "necklace order not supported");
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    const int depth = nk_depth(L);
    const std::vector<uint32_t> roots = nk_roots(L, depth);

    const size_t tab_words = (size_t)L * 2 * LS;
    const size_t off_init = nk_align((size_t)k * tab_words * 4);
    const size_t off_mod = nk_align(off_init + (size_t)k * 4);
    const size_t off_pinv = nk_align(off_mod + (size_t)k * 4);
    const size_t off_roots = nk_align(off_pinv + (size_t)k * 4);
    const size_t off_cnt = nk_align(off_roots + roots.size() * 4);
    const size_t off_acc = nk_align(off_cnt + (size_t)k * 4);
    const size_t off_status = nk_align(off_acc + (size_t)k * 8);
    const size_t total = nk_align(off_status + 16);
    Workspace *ws;
    st = workspace(&ws, total, total);
    if (st != PG_OK) return st;
    char *h = (char *)ws->host;
    char *d = (char *)ws->dev;
    std::memset(h, 0, off_roots);
    uint32_t *tab = (uint32_t *)h;
    for (int t = 0; t < k; t++) {
        const uint64_t p = primes[t], w = omegas[t] % p;
        std::vector<uint64_t> f(L);
        uint64_t e = 1;
        uint64_t sum = 0;
        for (int j = 0; j < L; j++) {
            f[j] = powmod_u64(w, e, p);
            sum += f[j];
            e = e * (uint64_t)g % (uint64_t)n;
        }
        uint32_t *tt = tab + (size_t)t * tab_words;
        for (int c = 0; c < L; c++)
            for (int r = 0; r < L; r++) {
                const uint32_t two = (uint32_t)(2 * f[(c - r + L) % L] % p);
                tt[(2 * c + 0) * LS + r] = two - (uint32_t)p;   // d_c = -1 -> +1: add 2f
                tt[(2 * c + 1) * LS + r] = 0u - two;            // d_c = +1 -> -1: subtract 2f
            }
        ((uint32_t *)(h + off_init))[t] = (uint32_t)(sum % p);
        ((uint32_t *)(h + off_mod))[t] = (uint32_t)p;
        ((uint32_t *)(h + off_pinv))[t] = neg_inv32((uint32_t)p);
    }
    std::memcpy(h + off_roots, roots.data(), roots.size() * 4);

    NeckArgs a;
    a.tabs = (const uint32_t *)d;
    a.init = (const uint32_t *)(d + off_init);
    a.moduli = (const uint32_t *)(d + off_mod);
    a.pinvs = (const uint32_t *)(d + off_pinv);
    a.roots = (const uint32_t *)(d + off_roots);
    a.nroots = (uint32_t)roots.size();
    a.depth = depth;
    a.counters = (unsigned int *)(d + off_cnt);
    a.acc = (unsigned long long *)(d + off_acc);
    a.abort_flag = abort_dev;
    a.status = (int *)(d + off_status);
    PG_CUDA(cudaMemcpyAsync(d, h, off_cnt, cudaMemcpyHostToDevice, ws->stream));
    PG_CUDA(cudaMemsetAsync(d + off_cnt, 0, total - off_cnt, ws->stream));
    PG_CUDA(launch_necklace(L, a, k, dev.sm_count, ws->stream));
    PG_CUDA(cudaMemcpyAsync(h + off_acc, d + off_acc, total - off_acc, cudaMemcpyDeviceToHost,
                            ws->stream));
    PG_CUDA(cudaStreamSynchronize(ws->stream));
    if (*(int *)(h + off_status)) return fail(PG_EABORT, "launch aborted by pg_abort()");
    const unsigned long long *acc = (const unsigned long long *)(h + off_acc);
    for (int t = 0; t < k; t++) {
        const uint64_t p = primes[t];
        uint64_t r = acc[t] % p;
        if (L >= 2) r = mulmod_u64(r, powmod_u64((1ull << 32) % p, (uint64_t)(L - 1), p), p);
        r = mulmod_u64(r, powmod_u64((p >> 1) + 1, (uint64_t)L, p), p);   // 2^-L
        out[t] = mulmod_u64(r, (uint64_t)n % p, p);
    }
    return PG_OK;
}

static bool odd_prime_order(int n) {
    if (n < 3 || !(n & 1)) return false;
    for (int d = 3; d * d <= n; d += 2)
        if (n % d == 0) return false;
    return true;
}

}  // namespace pg

// Representatives and covered sign words of the necklace quotient for an
// odd prime order 3 <= n < 64, counted on the host with the device walker.
// Replaces perm_c_ext.schur_necklace_orbit_stats (perm_c_omp.c:1062-1082).
extern "C" int pg_necklace_orbit_stats(int n, uint64_t *representatives, uint64_t *words) {
    using namespace pg;
    if (!representatives || !words) return fail(PG_EINVAL, "null argument");
    if (n >= 64 || !odd_prime_order(n))
        return fail(PG_ERANGE, "n must be an odd prime satisfying 3 <= n < 64");
    const int L = n - 1;
    struct Count {
        uint64_t reps = 0, words = 0;
        void operator()(uint64_t, uint32_t orbit) {
            reps++;
            words += orbit;
        }
    } c;
    const int depth = nk_depth(L);
    for (uint32_t r : nk_roots(L, depth)) nk_walk(r, depth, L, c);
    *representatives = c.reps;
    *words = c.words;
    return PG_OK;
}
