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
// The kernel does not dedupe weight-L/2 orbits: every necklace of weight
// < L/2 counts 2 * period (its rotations and its complement's), every
// necklace of weight L/2 counts period (its complement's necklace is visited
// on its own), which covers each of the 2^L words once without the
// complement test.
//
// GPU organisation: the host enumerates FKM subtree roots (the prefixes
// a[1..depth] of pre-necklaces, depth = L - F).  Each thread takes roots from
// a per-prime atomic counter and walks its subtree with the iterative FKM
// successor, which only moves the low F <= 24 bits of the word (32-bit
// branch-free steps, NkSubtreeWalker).  Candidates go to a small per-lane
// register queue; every round each lane evaluates one candidate and walks a
// few steps, so the product work stays uniform across the warp while the
// walk's varying step counts are absorbed by the queue.  A term's row sums
// come from a 256-entry byte table per prime in shared memory (the minor is
// circulant, so one table serves every byte position, read at a rotated row
// offset): rows of the bytes a subtree never changes, and of the rarely
// changing middle bytes, are kept summed in registers; a term reads one
// table row for its low byte and forms the product with the Montgomery
// chain of the Glynn residue kernel.  All primes run in one launch
// (grid.y = prime).  The walker is __host__ __device__:
// pg_necklace_orbit_stats counts the reference's rotation+complement orbits
// with the very same walker on the host.
#include "pg_internal.h"
#include "glynn_m32.cuh"

#include <cstring>
#include <vector>

namespace pg {

// Root: prefix bits a[1..depth] (a[1] most significant) in bits 0..31,
// Lyndon period of the prefix in bits 32..39.
constexpr int NK_MAX_DEPTH = 28;

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
__host__ __device__ __forceinline__ int nk_clz(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
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

// Orbit size of necklace w (period p) when w is the chosen representative
// of its rotation+complement orbit, else 0.  For weight L/2 the complement
// is in the same weight class and the smaller least rotation represents the
// orbit.  w, being a necklace, starts with its longest cyclic 0-run (length
// z); the complement's least rotation starts with the longest cyclic 1-run
// of w (length m).  m > z: the complement's rotation is smaller (reject);
// m < z: w is smaller (accept, orbit 2p); m == z: only the rotations of the
// complement that start at one of w's 1-runs of length z can be <= w, so
// those few are compared with w.  The top bit of w is 0, so no 1-run wraps
// around and plain shifts find the runs.
__host__ __device__ __forceinline__ uint32_t nk_orbit(uint64_t w, int p, int L) {
    const int weight = nk_popc(w), half = L / 2;
    if (weight < half) return 2u * p;
    if (weight > half) return 0;
    const int z = nk_clz(w) - (64 - L);    // w != 0 and starts with a 0
    uint64_t run = w;                      // bit x set: bits x .. x+j all ones
    for (int j = 1; j < z; j++) run &= run >> 1;
    if (!run) return 2u * p;               // m < z
    if (run & (run >> 1)) return 0;        // m > z
    const uint64_t mask = (1ull << L) - 1, c = ~w & mask;
    bool self = false;
    while (run) {                          // one bit per 1-run of length z
        const int x = nk_ctz(run);
        run &= run - 1;
        const int k = L - x - z;           // 1 <= k <= L - z: bit x+z-1 to the top
        const uint64_t r = ((c << k) | (c >> (L - k))) & mask;
        if (r < w) return 0;
        self |= r == w;
    }
    return self ? (uint32_t)p : 2u * p;
}

// Iterative FKM walker over one subtree (the pre-necklaces sharing a root's
// prefix, in lexicographic order).  step() looks at the current
// pre-necklace, reports it when it is an accepted representative, and moves
// to the next one; `live` drops when the subtree is exhausted.  Subtrees
// whose prefix is already heavier than L/2 are skipped whole.
struct NkWalker {
    uint64_t w;
    uint64_t free_mask;     // positions after the root prefix
    uint64_t divisors;      // bit d set when d divides L
    int p, L, depth;
    int last_p;             // period of the word the last step reported
    bool emit, live;

    __host__ __device__ __forceinline__ void init(int L_, int depth_) {
        L = L_;
        depth = depth_;
        free_mask = (1ull << (L - depth)) - 1;
        divisors = 0;
        for (int d = 1; d <= L; d++)
            if (L % d == 0) divisors |= 1ull << d;
        live = false;
    }
    __host__ __device__ __forceinline__ void start(uint64_t root) {
        p = (int)(root >> 32);
        const uint64_t prefix = root & 0xffffffffull;
        w = nk_extend(prefix >> (depth - p), p, L);
        emit = true;
        live = true;
    }
    // True with *word set (and last_p its period) when the visited
    // pre-necklace is a necklace of weight <= L/2; then moves on.
    __host__ __device__ __forceinline__ bool step(uint64_t *word) {
        const bool cand = emit && ((divisors >> p) & 1) && nk_popc(w) <= L / 2;
        if (cand) {
            *word = w;
            last_p = p;
        }
        const uint64_t free = ~w & free_mask;
        if (!free) {
            live = false;
            return cand;
        }
        const int b = nk_ctz(free);          // rightmost 0: position i = L - b
        const uint64_t pre = (w >> b) | 1ull;
        if (nk_popc(pre) > L / 2) {
            // every word below this prefix is heavier than L/2: fill the
            // tail with ones so the next successor moves left of it
            w = (pre << b) | ((1ull << b) - 1);
            emit = false;
        } else {
            p = L - b;
            w = nk_extend(pre, p, L);
            emit = true;
        }
        return cand;
    }
};

// Free bits of a subtree (the walker moves bits 0 .. F-1; the root prefix is
// bits F .. L-1).  Subtrees of at most 2^14 words keep the largest work item
// well below a thread's share; for long words the root count is held near
// 5 million (prefix depth 26) and later 28, so F grows up to 24 bits.
__host__ __device__ constexpr int nk_free_bits(int L) {
    return L <= 15 ? L - 1 : L <= 40 ? 14 : (L - 26 < 14 ? 14 : L - 26 > 24 ? 24 : L - 26);
}
__host__ __device__ constexpr int nk_depth_of(int L) { return L - nk_free_bits(L); }

// Queue entry of a candidate word: bits 0..23 the word's low 24 bits (the
// bytes a subtree changes), bits 24..29 its period p, bit 30 set when the
// word has weight L/2 and its orbit (2p, p or none) is still to be decided
// by the walker's resolve(), bit 31 the parity of its weight.  Without
// bit 30 the orbit is 2p.
constexpr uint32_t NK_HALF_FLAG = 1u << 30;
__host__ __device__ __forceinline__ uint32_t nk_entry(uint32_t low, int p, bool half, int parity) {
    return (low & 0xffffffu) | ((uint32_t)p << 24) | (half ? NK_HALF_FLAG : 0u) |
           ((uint32_t)parity << 31);
}
__host__ __device__ __forceinline__ int nk_popc32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}
__host__ __device__ __forceinline__ int nk_ctz32(uint32_t x) {   // x != 0
#ifdef __CUDA_ARCH__
    return __ffs((int)x) - 1;
#else
    return __builtin_ctz(x);
#endif
}

// Subtree walker for minor order L.  With F = nk_free_bits(L) and L >= 2F,
// the successor of a word sets its rightmost free 0 (bit b < F) and, the new
// period L - b being >= b, its periodic extension is a copy of the word's
// first b characters (the top b bits, inside the fixed prefix) into bits
// b-1..0.  Only b == 0 gives a period dividing L, so only those words (and
// the root's own first word) can be necklaces.  A step is a handful of
// 32-bit operations on the low word instead of 64-bit shifts and
// extensions.  Orders below 30 use the general walker.
template <int L, int F = nk_free_bits(L)>
struct NkSubtreeWalker {
    static constexpr bool FAST = L >= 30 && L >= 2 * F && F <= 24;
    static constexpr int HALF = L / 2;
    NkWalker g;
    uint64_t high;   // bits 32..L-1 (fixed within the subtree)
    uint32_t lo;     // bits 0..31 of the current word
    uint32_t top;    // the word's top 24 bits, a[1..24]
    int wh, p;
    bool emit, live;

    __host__ __device__ __forceinline__ void init() {
        g.init(L, L - F);
        live = false;
    }
    __host__ __device__ __forceinline__ void start(uint64_t root) {
        g.start(root);
        live = true;
        if constexpr (FAST) {
            const uint64_t w = g.w;
            high = w & ~0xffffffffull;
            lo = (uint32_t)w;
            top = (uint32_t)(w >> (L - 24)) & 0xffffffu;
            wh = nk_popc(high);
            p = g.p;
            emit = L % p == 0;
        }
    }
    // the current word (its bytes from F up never change within the subtree)
    __host__ __device__ __forceinline__ uint64_t word() const {
        if constexpr (FAST) return high | lo;
        return g.w;
    }
    // Weight the kernel gives a candidate: 2p below weight L/2 (the word's
    // rotations and those of its complement, which is heavier than L/2 and
    // never visited), p at weight L/2 (its rotations only: the complement's
    // necklace has weight L/2 too and is visited on its own, and a
    // self-complementary necklace covers both halves by itself).  Every sign
    // word is covered exactly once and no dedupe test is needed.
    __host__ __device__ __forceinline__ static uint32_t cover(uint32_t e) {
        const uint32_t q = (e >> 24) & 0x3f;
        return (e & NK_HALF_FLAG) ? q : 2u * q;
    }
    // Orbit size under rotation and complement when the candidate represents
    // its orbit, else 0 (rivin-perm's counting, perm_c_omp.c:104-121).
    __host__ __device__ __forceinline__ uint32_t exact(uint32_t e) const {
        const int q = (int)((e >> 24) & 0x3f);
        if (!(e & NK_HALF_FLAG)) return 2u * q;
        return nk_orbit((word() & ~0xffffffull) | (e & 0xffffffu), q, L);
    }
    // Visits the current pre-necklace and moves to the next one.  Returns
    // true with *entry set when the visited word is a candidate (a necklace
    // of weight <= L/2); weight-L/2 candidates carry NK_HALF_FLAG.
    __host__ __device__ __forceinline__ bool step(uint32_t *entry) {
        if constexpr (!FAST) {
            uint64_t w = 0;
            const bool cand = g.step(&w);
            live = g.live;
            if (cand) *entry = nk_entry((uint32_t)w, g.last_p, nk_popc(w) == HALF, nk_popc(w) & 1);
            return cand;
        } else {
            // visit: the word is a necklace when emit is set (its period
            // divides L); it is a candidate unless heavier than L/2
            const int weight = wh + nk_popc32(lo);
            const bool cand = emit && weight <= HALF;
            *entry = nk_entry(lo, p, weight == HALF, weight & 1);
            // successor, branch-free: rightmost free 0 at bit b becomes 1 and
            // bits below b copy a[1..b]; a prefix heavier than L/2 instead
            // fills bits below b with ones so the next step moves past it
            const uint32_t free = ~lo & ((1u << F) - 1);
            live = free != 0;
            const int b = nk_ctz32(free | (1u << F));
            const uint32_t pre = (lo >> b) | 1u;
            const bool heavy = wh + nk_popc32(pre) > HALF;
            const uint32_t tail = heavy ? (1u << b) - 1 : top >> (24 - b);
            lo = (pre << b) | tail;
            p = heavy ? p : L - b;
            emit = !heavy && b == 0;
            return cand;
        }
    }
};

// Host: FKM subtree roots at prefix depth `depth`, prefix weight <= L/2
// (perm_c_omp.c:375-402 collects subtree states the same way for its
// CPU threads).
static void nk_roots_rec(std::vector<uint64_t> &out, uint8_t *a, int t, int period,
                         int weight, uint32_t prefix, int L, int depth) {
    if (t > depth) {
        out.push_back(prefix | ((uint64_t)period << 32));
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

static std::vector<uint64_t> nk_roots(int L, int depth) {
    std::vector<uint64_t> out;
    uint8_t a[NK_MAX_DEPTH + 2] = {0};
    nk_roots_rec(out, a, 1, 1, 0, 0, L, depth);
    return out;
}

static int nk_depth(int L) { return nk_depth_of(L); }

// Chunk table row stride in words: a multiple of 4 with an odd count of
// 16-byte units, so 128-bit reads of different rows spread over the banks.
__host__ __device__ constexpr int nk_stride(int L) {
    return ((L + 3) / 4 % 2 == 1) ? (L + 3) / 4 * 4 : (L + 3) / 4 * 4 + 4;
}

// Moduli of the necklace kernel: a row sum is summed lazily from two terms
// below p (< 2p), and the Montgomery chain stays below 2p as long as
// 4p < 2^32: NECKLACE_PRIME_LIMIT = 2^30.  The wide form (W) takes odd
// moduli up to 2^32 (the reference's 32-bit pseudo-Mersenne primes) and
// keeps every value fully reduced, with 33-bit intermediate sums
// (m32w_addmod, m32w_redc_mul).
constexpr uint64_t NK_PRIME_LIMIT = NECKLACE_PRIME_LIMIT;

struct NeckArgs {
    // [k][256][LS]: entry (v, x) = sum over set bits t of the byte v of
    // -2 f[(L - 1 - t - x) mod L] mod p, i.e. the change of row x's sum when
    // the bits of v in byte 0 of the word flip from + to -.  Byte j of the
    // word reads row x = (r + 8j) mod L (the minor is circulant).
    const uint32_t *tabs;
    const uint32_t *s0;       // [k] row sum of the all-plus word (equal for all rows)
    const uint32_t *moduli;
    const uint32_t *pinvs;
    const uint64_t *roots;
    uint32_t nroots;
    unsigned int *counters;   // [k] root counters (zeroed)
    unsigned long long *acc;  // [k] (zeroed)
    volatile const int *abort_flag;
    int *status;
};

constexpr int NK_CHAINS = 4;      // Montgomery chains per term

template <int L, bool W = false>
struct NeckLane {
    static constexpr int LS = nk_stride(L);
    static constexpr int NCH = (L + 7) / 8;                     // bytes of an L-bit word
    static constexpr int NLOW = (nk_free_bits(L) + 7) / 8;      // bytes a subtree changes
    static constexpr int V = (L % 4 == 0) ? 4 : 2;              // table read width
    // s0 plus the contributions of every byte except byte 0, for the bytes
    // 1..NLOW-1 recorded in `cur` (bits 8..23 of a word), in [0, p).  Words
    // of a subtree come in lexicographic order, so those bytes change only
    // every few dozen words and a term reads one table row (byte 0).
    uint32_t hm[L];
    uint32_t cur;
    uint32_t p, pinv;
    unsigned long long acc;   // sum of signed terms, odd-weight ones as 256p - v
    uint32_t count;

    // Row sums of the bytes a subtree never changes (bytes 1..NLOW-1 taken
    // as 0).  Runs once per subtree.
    __device__ __forceinline__ void set_high(const uint32_t *tab, uint32_t s0, uint64_t w) {
#pragma unroll
        for (int r = 0; r < L; r++) hm[r] = s0;
#pragma unroll
        for (int j = NLOW; j < NCH; j++) {
            const uint32_t *t = tab + ((w >> (8 * j)) & 0xff) * LS;
#pragma unroll
            for (int r = 0; r < L; r++) {
                const uint32_t d = t[(r + 8 * j) % L];
                hm[r] = W ? m32w_addmod(hm[r], d, p) : m32_addmod(hm[r], d - p, p);
            }
        }
        cur = 0;
    }

    // Brings hm to the bytes 1..NLOW-1 of entry e: for each byte that
    // differs, add table row (r + 8j) mod L of the new value and subtract
    // the old one.
    __device__ __forceinline__ void follow(const uint32_t *tab, uint32_t e) {
        const uint32_t nw = (e >> 8) & 0xffffu;
        if (nw == cur) return;
#pragma unroll
        for (int j = 1; j < NLOW; j++) {
            const uint32_t ov = (cur >> (8 * (j - 1))) & 0xff, nv = (nw >> (8 * (j - 1))) & 0xff;
            if (ov == nv) continue;
            const uint32_t *to = tab + ov * LS, *tn = tab + nv * LS;
#pragma unroll
            for (int r = 0; r < L; r++) {
                const uint32_t x = tn[(r + 8 * j) % L], y = to[(r + 8 * j) % L];
                const uint32_t d = x >= y ? x - y : x - y + p;     // (x - y) mod p
                hm[r] = W ? m32w_addmod(hm[r], d, p) : m32_addmod(hm[r], d - p, p);
            }
        }
        cur = nw;
    }

    // Term of one queued word: row r's sum is hm[r] plus table row r of
    // byte 0 (< 2p).
    __device__ __forceinline__ void eval(const uint32_t *tab, uint32_t e, uint32_t orbit) {
        const uint32_t *t0 = tab + (e & 0xff) * LS;
        // narrow: lazy sums below 2p and the chain of the residue kernel;
        // wide: fully reduced sums and products
        const auto add2 = [&](uint32_t x, uint32_t y) {
            return W ? m32w_addmod(x, y, p) : x + y;
        };
        const auto mul = [&](uint32_t x, uint32_t y) {
            return W ? m32w_redc_mul(x, y, p, pinv) : m32_redc_mul(x, y, p, pinv);
        };
        uint32_t prod;
        if constexpr (L >= 8) {
            // C independent Montgomery chains (ILP), joined by a pairwise
            // tree: (L - C) + (C - 1) = L - 1 reductions in all.  Row sums and
            // chain values stay below 2p.
            constexpr int C = L >= 2 * NK_CHAINS ? NK_CHAINS : 4;
            uint32_t ch[C];
#pragma unroll
            for (int q = 0; q < L / V; q++) {
                uint32_t sr[V];
                if constexpr (V == 4) {
                    const uint4 x = *reinterpret_cast<const uint4 *>(t0 + 4 * q);
                    sr[0] = add2(hm[4 * q], x.x); sr[1] = add2(hm[4 * q + 1], x.y);
                    sr[2] = add2(hm[4 * q + 2], x.z); sr[3] = add2(hm[4 * q + 3], x.w);
                } else {
                    const uint2 x = *reinterpret_cast<const uint2 *>(t0 + 2 * q);
                    sr[0] = add2(hm[2 * q], x.x); sr[1] = add2(hm[2 * q + 1], x.y);
                }
#pragma unroll
                for (int i = 0; i < V; i++) {
                    const int r = V * q + i;
                    if (r < C) ch[r] = sr[i];
                    else ch[r % C] = mul(ch[r % C], sr[i]);
                }
            }
#pragma unroll
            for (int w = 1; w < C; w *= 2)
#pragma unroll
                for (int i = 0; i + w < C; i += 2 * w)
                    ch[i] = mul(ch[i], W ? ch[i + w] : __viaddmin_u32(ch[i + w], 0u - p, ch[i + w]));
            prod = ch[0];
        } else {
            // L < 8: one byte; reduce each row sum and chain serially
            prod = 0;
#pragma unroll
            for (int r = 0; r < L; r++) {
                uint32_t sr = add2(hm[r], t0[r]);
                if (!W) sr = __viaddmin_u32(sr, 0u - p, sr);
                prod = r == 0 ? sr : mul(prod, sr);
            }
        }
        // prod * orbit < 2p * 120 < 256p: an odd-weight term adds 256p - v
        const unsigned long long v = (unsigned long long)prod * orbit;
        acc += (e >> 31) ? ((unsigned long long)p << 8) - v : v;
        if (++count == (1u << 20)) {     // each addend < 2^40: reduce long before 2^64
            acc %= p;
            count = 0;
        }
    }
};

// Per-lane queue of accepted words, in registers (compile-time indices only).
template <int QN>
struct NkQueue {
    uint32_t q[QN];
    int n = 0;
    __device__ __forceinline__ void push(uint32_t e) {
#pragma unroll
        for (int i = 0; i < QN; i++) q[i] = (i == n) ? e : q[i];
        n++;
    }
    __device__ __forceinline__ uint32_t pop() {
        const uint32_t e = q[0];
#pragma unroll
        for (int i = 0; i + 1 < QN; i++) q[i] = q[i + 1];
        n--;
        return e;
    }
};

constexpr int NK_QUEUE = 4;        // accepted words a lane may hold
constexpr int NK_WALK_STEPS = 3;   // walker steps per evaluation (about 2.5 steps per word)

// Resident blocks per SM requested from ptxas for orders up to 42: three
// (80 registers, a few bytes of spill) beat two by 4-11 % on S_37..S_43,
// the walk's latency being hidden by more warps.  0: no request.
#ifndef PG_NK_MIN_BLOCKS
#define PG_NK_MIN_BLOCKS 3
#endif
__host__ __device__ constexpr int nk_min_blocks(int L) {
    return PG_NK_MIN_BLOCKS > 0 && L <= 42 ? PG_NK_MIN_BLOCKS : 1;
}

template <int L, bool W>
__global__ void __launch_bounds__(256, nk_min_blocks(L)) necklace_m32_kernel(NeckArgs a) {
    constexpr int LS = nk_stride(L);
    extern __shared__ uint4 nsm[];
    const int k = blockIdx.y;
    {
        const uint4 *g = reinterpret_cast<const uint4 *>(a.tabs + (size_t)k * 256 * LS);
        for (int i = threadIdx.x; i < 256 * LS / 4; i += blockDim.x) nsm[i] = g[i];
    }
    __syncthreads();
    const uint32_t *tab = reinterpret_cast<const uint32_t *>(nsm);
    NeckLane<L, W> lane;
    lane.p = a.moduli[k];
    lane.pinv = a.pinvs[k];
    lane.acc = 0;
    lane.count = 0;
    const uint32_t s0 = a.s0[k];
    NkSubtreeWalker<L> wk;
    wk.init();
    NkQueue<NK_QUEUE> queue;
    bool finished = false, aborted = false;
    // Each round: a lane whose subtree is done and whose queue is empty takes
    // the next root; then every lane evaluates one queued candidate (entry 0,
    // of weight 0, when its queue is empty) and walks NK_WALK_STEPS steps
    // (skipped while its queue is full).  The evaluation and the steps are
    // independent straight-line code, so the IMAD chains of the product and
    // the ALU work of the walk interleave.  Queued words always belong to
    // the subtree whose high bytes are in lane.hm.
    for (;;) {
        if (!wk.live && queue.n == 0 && !finished) {
            const unsigned int r = atomicAdd(a.counters + k, 1u);
            if (r >= a.nroots) {
                finished = true;
            } else if (*a.abort_flag) {
                finished = aborted = true;
            } else {
                wk.start(a.roots[r]);
                lane.set_high(tab, s0, wk.word());
            }
        }
        if (__all_sync(0xffffffffu, finished)) break;
        const bool have = queue.n > 0;
        const uint32_t e = have ? queue.pop() : 0u;
        if constexpr (NeckLane<L>::NLOW > 1) {
            if (have) lane.follow(tab, e);
        }
        lane.eval(tab, e, NkSubtreeWalker<L>::cover(e));
#pragma unroll
        for (int st = 0; st < NK_WALK_STEPS; st++) {
            uint32_t entry;
            const bool go = wk.live && queue.n < NK_QUEUE;
            if (go && wk.step(&entry)) queue.push(entry);
        }
    }
    const uint32_t p = lane.p;
    unsigned long long v = lane.acc % p;
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

// Minor orders L = n - 1 of the odd primes 3 .. 53 (59 and 61 would need
// more than 2^28 subtree roots or four changing bytes; their counts are far
// beyond any run anyway).
#define PG_NK_ORDERS(X) X(2) X(4) X(6) X(10) X(12) X(16) X(18) X(22) X(28) X(30) \
                        X(36) X(40) X(42) X(46) X(52)
// Orders with the wide-modulus kernel (odd moduli 2^30 <= p < 2^32): the
// orders of the automatic necklace dispatch (n >= 37).
#define PG_NK_WIDE_ORDERS(X) X(36) X(40) X(42) X(46) X(52)

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

bool necklace_wide_supported(int n) {
    switch (n - 1) {
#define PG_NK_YES(LL) case LL:
        PG_NK_WIDE_ORDERS(PG_NK_YES)
#undef PG_NK_YES
        return true;
    default:
        return false;
    }
}

template <int L, bool W>
static cudaError_t launch_necklace_t(const NeckArgs &a, int k, int sm_count, cudaStream_t s) {
    const size_t smem = (size_t)256 * nk_stride(L) * 4;
    cudaError_t e = cudaFuncSetAttribute(necklace_m32_kernel<L, W>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, necklace_m32_kernel<L, W>, 256,
                                                      smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const int bpm = (per_sm * sm_count + k - 1) / k;
    dim3 grid(bpm, k);
    necklace_m32_kernel<L, W><<<grid, 256, smem, s>>>(a);
    return cudaGetLastError();
}

static cudaError_t launch_necklace(int L, bool wide, const NeckArgs &a, int k, int sm_count,
                                   cudaStream_t s) {
    if (wide) {
        switch (L) {
#define PG_NK_CASE(LL) case LL: return launch_necklace_t<LL, true>(a, k, sm_count, s);
            PG_NK_WIDE_ORDERS(PG_NK_CASE)
#undef PG_NK_CASE
        default:
            return cudaErrorInvalidValue;
        }
    }
    switch (L) {
#define PG_NK_CASE(LL) case LL: return launch_necklace_t<LL, false>(a, k, sm_count, s);
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

// One launch over k primes of one width (wide: 2^30 <= p < 2^32).
static int necklace_group(int n, int g, const std::vector<uint64_t> &roots,
                          const uint64_t *primes, const uint64_t *omegas, int k, bool wide,
                          uint64_t *out) {
    const int L = n - 1, LS = nk_stride(L);
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;

    const size_t tab_words = (size_t)256 * LS;
    const size_t off_s0 = nk_align((size_t)k * tab_words * 4);
    const size_t off_mod = nk_align(off_s0 + (size_t)k * 4);
    const size_t off_pinv = nk_align(off_mod + (size_t)k * 4);
    const size_t off_roots = nk_align(off_pinv + (size_t)k * 4);
    const size_t off_cnt = nk_align(off_roots + roots.size() * 8);
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
        // circulant minor in primitive-root order: M[r][c] = f[(c - r) mod L]
        std::vector<uint64_t> f(L);
        uint64_t e = 1, sum = 0;
        for (int j = 0; j < L; j++) {
            f[j] = powmod_u64(w, e, p);
            sum += f[j];
            e = e * (uint64_t)g % (uint64_t)n;
        }
        // byte table: bit b of the word is column L - 1 - b; flipping it from
        // + to - changes row x's sum by -2 f[(L - 1 - b - x) mod L]
        uint32_t *tt = tab + (size_t)t * tab_words;
        for (int v = 1; v < 256; v++) {
            const int b = __builtin_ctz((unsigned)v);
            const uint32_t *prev = tt + (size_t)(v & (v - 1)) * LS;
            uint32_t *row = tt + (size_t)v * LS;
            for (int x = 0; x < L; x++) {
                const int c = (((L - 1 - b - x) % L) + L) % L;
                const uint64_t delta = (p - 2 * f[c] % p) % p;
                row[x] = (uint32_t)((prev[x] + delta) % p);
            }
        }
        ((uint32_t *)(h + off_s0))[t] = (uint32_t)(sum % p);
        ((uint32_t *)(h + off_mod))[t] = (uint32_t)p;
        ((uint32_t *)(h + off_pinv))[t] = neg_inv32((uint32_t)p);
    }
    std::memcpy(h + off_roots, roots.data(), roots.size() * 8);

    NeckArgs a;
    a.tabs = (const uint32_t *)d;
    a.s0 = (const uint32_t *)(d + off_s0);
    a.moduli = (const uint32_t *)(d + off_mod);
    a.pinvs = (const uint32_t *)(d + off_pinv);
    a.roots = (const uint64_t *)(d + off_roots);
    a.nroots = (uint32_t)roots.size();
    a.counters = (unsigned int *)(d + off_cnt);
    a.acc = (unsigned long long *)(d + off_acc);
    a.abort_flag = abort_dev;
    a.status = (int *)(d + off_status);
    PG_CUDA(cudaMemcpyAsync(d, h, off_cnt, cudaMemcpyHostToDevice, ws->stream));
    PG_CUDA(cudaMemsetAsync(d + off_cnt, 0, total - off_cnt, ws->stream));
    PG_CUDA(launch_necklace(L, wide, a, k, dev.sm_count, ws->stream));
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

// n * per(circulant Schur minor) mod primes[t] = perm(S_n) mod primes[t],
// for prime n with necklace_supported(n), odd primes[t] < NK_PRIME_LIMIT (or
// < 2^32 when necklace_wide_supported(n)) and omegas[t]^n == 1 (mod
// primes[t]).  Narrow and wide moduli run as two launches.
int schur_necklace_residues(int n, const uint64_t *primes, const uint64_t *omegas, int k,
                            uint64_t *out) {
    if (k <= 0) return PG_OK;
    const int g = primitive_root_of_prime(n);
    if (g < 0 || !necklace_supported(n)) return fail(PG_EINTERNAL, "necklace order not supported");
    std::vector<uint64_t> pw[2], ww[2], res[2];
    std::vector<int> idx[2];
    for (int t = 0; t < k; t++) {
        const bool wide = primes[t] >= NK_PRIME_LIMIT;
        if (!(primes[t] & 1) || primes[t] >= NECKLACE_WIDE_PRIME_LIMIT ||
            (wide && !necklace_wide_supported(n)))
            return fail(PG_EINTERNAL, "necklace modulus must be odd and below 2^30 "
                                      "(2^32 for the wide orders)");
        pw[wide].push_back(primes[t]);
        ww[wide].push_back(omegas[t]);
        idx[wide].push_back(t);
    }
    const std::vector<uint64_t> roots = nk_roots(n - 1, nk_depth(n - 1));
    for (int w = 0; w < 2; w++) {
        if (pw[w].empty()) continue;
        res[w].assign(pw[w].size(), 0);
        const int st = necklace_group(n, g, roots, pw[w].data(), ww[w].data(),
                                      (int)pw[w].size(), w == 1, res[w].data());
        if (st != PG_OK) return st;
        for (size_t i = 0; i < idx[w].size(); i++) out[idx[w][i]] = res[w][i];
    }
    return PG_OK;
}

static bool odd_prime_order(int n) {
    if (n < 3 || !(n & 1)) return false;
    for (int d = 3; d * d <= n; d += 2)
        if (n % d == 0) return false;
    return true;
}

// Representatives and covered words, counted with the kernel's walker.
template <int L, int F = nk_free_bits(L)>
static void count_orbits(uint64_t *reps, uint64_t *covered) {
    NkSubtreeWalker<L, F> wk;
    wk.init();
    for (uint64_t r : nk_roots(L, L - F)) {
        wk.start(r);
        while (wk.live) {
            uint32_t entry;
            if (!wk.step(&entry)) continue;
            const uint32_t orb = wk.exact(entry);
            if (orb) {
                ++*reps;
                *covered += orb;
            }
        }
    }
}

}  // namespace pg

// Representatives and covered sign words of the necklace quotient for an
// odd prime order 3 <= n < 64, counted on the host with the kernel's walker.
// Replaces perm_c_ext.schur_necklace_orbit_stats (perm_c_omp.c:1062-1082).
extern "C" int pg_necklace_orbit_stats(int n, uint64_t *representatives, uint64_t *words) {
    using namespace pg;
    if (!representatives || !words) return fail(PG_EINVAL, "null argument");
    if (n >= 64 || !odd_prime_order(n))
        return fail(PG_ERANGE, "n must be an odd prime satisfying 3 <= n < 64");
    uint64_t reps = 0, covered = 0;
    switch (n - 1) {
#define PG_NK_COUNT(LL) case LL: count_orbits<LL>(&reps, &covered); break;
        PG_NK_ORDERS(PG_NK_COUNT)
#undef PG_NK_COUNT
    default: {
        // orders without a kernel (59, 61): the general walker at depth 26
        const int L = n - 1;
        NkWalker g;
        g.init(L, 26);
        for (uint64_t r : nk_roots(L, 26)) {
            g.start(r);
            while (g.live) {
                uint64_t w;
                if (!g.step(&w)) continue;
                const uint32_t orb = nk_orbit(w, g.last_p, L);
                if (orb) {
                    reps++;
                    covered += orb;
                }
            }
        }
    }
    }
    *representatives = reps;
    *words = covered;
    return PG_OK;
}
