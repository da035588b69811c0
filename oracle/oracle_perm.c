/*
 * CPU oracle for the exact-permanent hot path.  TEST INFRASTRUCTURE ONLY:
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
 * library as the checker / CPU baseline; the GPU product path never calls it.
 *
 * Plain C99 + OpenMP restatement of the reference algorithms (rivin-perm):
 *
 *   or_permanent_mod_p      perm_c_omp.c:846-854  (Glynn iff n>=4, p odd and
 *                           p <= 3037000499, else Ryser) with entries reduced
 *                           mod p first as at perm_c_omp.c:911
 *   or_glynn_mod_p          perm_c_omp.c:510-554 serial / 556-639 parallel
 *                           (contiguous Gray blocks, closed-form block start)
 *   or_ryser_mod_p          perm_c_omp.c:666-823
 *   or_schur_mod_p          perm_c_omp.c:942-1060 without the necklace
 *                           quotient (same residue: n * per(minor) for the
 *                           (n-1)x(n-1) minor w^((r+1)(c+1)), Glynn on it)
 *   or_binary_mod_p         perm_binary_omp.c:386-519 contract (odd prime
 *                           p > n) evaluated with the plain Glynn sum; the
 *                           reference's ratio/Montgomery update is an
 *                           implementation detail that yields the same residue
 *   or_glynn_f64            perm_parallel_cuda.cu:68-209 (+ Kahan per block,
 *                           ldexp(-(n-1)) at :405), also returning sum |terms|
 *   or_glynn_f64_grad       d per / d a_ij = per(A without row i, column j),
 *                           evaluated by Glynn on every minor (small n only)
 *   or_mod3_range           Ryser mod 3 with bit-sliced F_3 row sums over a
 *                           range of the 2^n Gray-ordered subsets
 *                           (perm_mod3_omp.c:54-160, perm_mod3.py:143-228)
 *   or_affine_mod_p         coefficients of per(C + x L) mod an odd modulus:
 *                           the fixed-sign Glynn sum with affine row sums and
 *                           the product of n linear factors per state
 *                           (perm_polynomial.py:268-329, native engine
 *                           perm_polynomial_omp.c:434-486, 612-636, 681-779)
 *
 * Parity of this restatement is pinned against the reference's own compiled
 * extensions and golden values in tests/golden (see tests/test_oracle_pins.py).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

static inline int64_t norm_mod(int64_t v, int64_t p) {
    int64_t r = v % p;
    return r < 0 ? r + p : r;
}
static inline int64_t add_mod(int64_t a, int64_t b, int64_t p) {
    return a >= p - b ? a - (p - b) : a + b;
}
static inline int64_t sub_mod(int64_t a, int64_t b, int64_t p) {
    return a >= b ? a - b : p - (b - a);
}
static inline int64_t mul_mod(int64_t a, int64_t b, int64_t p) {
    return (int64_t)(((u128)(uint64_t)a * (u128)(uint64_t)b) % (u128)(uint64_t)p);
}
static int64_t pow_mod(int64_t b, uint64_t e, int64_t p) {
    int64_t r = 1 % p;
    while (e) {
        if (e & 1) r = mul_mod(r, b, p);
        b = mul_mod(b, b, p);
        e >>= 1;
    }
    return r;
}

int or_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Largest modulus whose residue products fit a signed 64-bit product: the
 * reference multiplies row sums with a plain 64-bit (a * b) % p up to it and
 * with 128-bit arithmetic above (perm_c_omp.c:36-47 selector). */
#define OR_DIRECT_MUL_LIMIT INT64_C(3037000499)

static inline int64_t row_product(const int64_t *rs, int n, int64_t p) {
    int64_t prod = 1 % p;
    if (p <= OR_DIRECT_MUL_LIMIT) {
        for (int r = 0; r < n; r++) prod = (prod * rs[r]) % p;
    } else {
        for (int r = 0; r < n; r++) prod = mul_mod(prod, rs[r], p);
    }
    return prod;
}

/* Glynn over states [lo, hi) of the 2^(n-1) fixed-last-sign Gray walk.
 * Entries of m are in [0, p).  Returns the signed partial sum mod p. */
static int64_t glynn_block(const int64_t *m, int n, int64_t p,
                           uint64_t lo, uint64_t hi) {
    int64_t rs[64];
    for (int r = 0; r < n; r++) {
        int64_t s = 0;
        for (int c = 0; c < n; c++) s = add_mod(s, m[r * n + c], p);
        rs[r] = s;
    }
    uint64_t g = lo ^ (lo >> 1);
    for (int c = 0; c < n - 1; c++)
        if ((g >> c) & 1)
            for (int r = 0; r < n; r++)
                rs[r] = sub_mod(rs[r], add_mod(m[r * n + c], m[r * n + c], p), p);
    int sign = (__builtin_popcountll(g) & 1) ? -1 : 1;
    int64_t acc = 0;
    for (uint64_t s = lo; s < hi; s++) {
        if (s != lo) {
            int c = __builtin_ctzll(s);
            uint64_t gs = s ^ (s >> 1);
            int sub = (int)((gs >> c) & 1);
            for (int r = 0; r < n; r++) {
                int64_t t = add_mod(m[r * n + c], m[r * n + c], p);
                rs[r] = sub ? sub_mod(rs[r], t, p) : add_mod(rs[r], t, p);
            }
            sign = -sign;
        }
        const int64_t prod = row_product(rs, n, p);
        acc = sign < 0 ? sub_mod(acc, prod, p) : add_mod(acc, prod, p);
    }
    return acc;
}

/* Glynn mod odd p, entries already in [0, p); threads <= 1 is serial. */
int64_t or_glynn_mod_p(const int64_t *m, int n, int64_t p, int threads) {
    if (n == 0) return 1 % p;
    if (n == 1) return m[0] % p;
    uint64_t states = 1ULL << (n - 1);
    int64_t total = 0;
    if (threads <= 1 || n <= 16) {
        total = glynn_block(m, n, p, 0, states);
    } else {
#pragma omp parallel num_threads(threads)
        {
            int t = 0, nt = 1;
#ifdef _OPENMP
            t = omp_get_thread_num();
            nt = omp_get_num_threads();
#endif
            uint64_t blk = (states + (uint64_t)nt - 1) / (uint64_t)nt;
            uint64_t lo = (uint64_t)t * blk, hi = lo + blk;
            if (hi > states) hi = states;
            int64_t part = lo < hi ? glynn_block(m, n, p, lo, hi) : 0;
#pragma omp critical
            total = add_mod(total, part, p);
        }
    }
    int64_t inv2 = (p >> 1) + 1;
    return mul_mod(total, pow_mod(inv2, (uint64_t)(n - 1), p), p);
}

/* Partial Glynn sum over states [lo, hi) (no 2^(1-n) scaling), split into
 * contiguous blocks over `threads` OpenMP threads — the CPU-baseline sample
 * of perm_c_omp.c:556-639 restricted to a state range. */
int64_t or_glynn_range_mod_p(const int64_t *a, int n, int64_t p, uint64_t lo,
                             uint64_t hi, int threads) {
    if (n < 2 || p < 3 || !(p & 1) || lo >= hi) return 0;
    int64_t *m = (int64_t *)malloc((size_t)n * n * sizeof(int64_t));
    if (!m) return -1;
    for (int i = 0; i < n * n; i++) m[i] = norm_mod(a[i], p);
    int64_t total = 0;
    uint64_t span = hi - lo;
#pragma omp parallel num_threads(threads > 1 ? threads : 1)
    {
        int t = 0, nt = 1;
#ifdef _OPENMP
        t = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        uint64_t blk = (span + (uint64_t)nt - 1) / (uint64_t)nt;
        uint64_t b0 = lo + (uint64_t)t * blk, b1 = b0 + blk;
        if (b1 > hi) b1 = hi;
        int64_t part = b0 < b1 ? glynn_block(m, n, p, b0, b1) : 0;
#pragma omp critical
        total = add_mod(total, part, p);
    }
    free(m);
    return total;
}

static int64_t ryser_block(const int64_t *m, int n, int64_t p,
                           uint64_t lo, uint64_t hi) {
    int64_t rs[64];
    if (lo == 0) lo = 1;
    if (lo >= hi) return 0;
    for (int r = 0; r < n; r++) rs[r] = 0;
    uint64_t g = lo ^ (lo >> 1);
    for (int c = 0; c < n; c++)
        if ((g >> c) & 1)
            for (int r = 0; r < n; r++) rs[r] = add_mod(rs[r], m[r * n + c], p);
    int sign = (__builtin_popcountll(g) & 1) ? -1 : 1;
    int64_t acc = 0;
    for (uint64_t s = lo; s < hi; s++) {
        if (s != lo) {
            int c = __builtin_ctzll(s);
            uint64_t gs = s ^ (s >> 1);
            int add = (int)((gs >> c) & 1);
            for (int r = 0; r < n; r++)
                rs[r] = add ? add_mod(rs[r], m[r * n + c], p)
                            : sub_mod(rs[r], m[r * n + c], p);
            sign = -sign;
        }
        int64_t prod = 1 % p;
        for (int r = 0; r < n; r++) prod = mul_mod(prod, rs[r], p);
        acc = sign < 0 ? sub_mod(acc, prod, p) : add_mod(acc, prod, p);
    }
    return acc;
}

/* Ryser mod any p >= 1, entries in [0, p). */
int64_t or_ryser_mod_p(const int64_t *m, int n, int64_t p, int threads) {
    if (n == 0) return 1 % p;
    if (n == 1) return m[0] % p;
    uint64_t states = 1ULL << n;
    int64_t total = 0;
    if (threads <= 1 || n <= 16) {
        total = ryser_block(m, n, p, 0, states);
    } else {
#pragma omp parallel num_threads(threads)
        {
            int t = 0, nt = 1;
#ifdef _OPENMP
            t = omp_get_thread_num();
            nt = omp_get_num_threads();
#endif
            uint64_t blk = (states + (uint64_t)nt - 1) / (uint64_t)nt;
            uint64_t lo = (uint64_t)t * blk, hi = lo + blk;
            if (hi > states) hi = states;
            int64_t part = lo < hi ? ryser_block(m, n, p, lo, hi) : 0;
#pragma omp critical
            total = add_mod(total, part, p);
        }
    }
    if (n & 1) total = total == 0 ? 0 : p - total;
    return total;
}

/* Generic selector: raw int64 entries, any modulus p >= 1 (p < 2^63). */
int64_t or_permanent_mod_p(const int64_t *a, int n, int64_t p, int threads) {
    if (p <= 0 || n < 0 || n >= 64) return -1;
    if (n == 0) return 1 % p;
    int64_t *m = (int64_t *)malloc((size_t)n * n * sizeof(int64_t));
    if (!m) return -1;
    for (int i = 0; i < n * n; i++) m[i] = norm_mod(a[i], p);
    int64_t r;
    if (n == 1) r = m[0];
    else if (n >= 4 && p > 1 && (p & 1) && p <= INT64_C(3037000499))
        r = or_glynn_mod_p(m, n, p, threads);
    else
        r = or_ryser_mod_p(m, n, p, threads);
    free(m);
    return r;
}

/* perm(S_n) mod p for odd n, omega^n == 1, odd p (the Glynn branch of the
 * reference); other preconditions use the full matrix with Ryser. */
int64_t or_schur_mod_p(int n, int64_t omega, int64_t p, int threads) {
    if (n < 0 || n >= 64 || p <= 0) return -1;
    if (n <= 1) return 1 % p;
    if (p == 1) return 0;
    int64_t w = norm_mod(omega, p);
    int64_t r;
    if (n >= 3 && (n & 1) && (p & 1) && pow_mod(w, (uint64_t)n, p) == 1 % p) {
        int k = n - 1;
        int64_t *m = (int64_t *)malloc((size_t)k * k * sizeof(int64_t));
        if (!m) return -1;
        int64_t wj = w;
        for (int row = 0; row < k; row++) {
            int64_t pw = wj;
            for (int c = 0; c < k; c++) {
                m[row * k + c] = pw;
                pw = mul_mod(pw, wj, p);
            }
            wj = mul_mod(wj, w, p);
        }
        r = or_glynn_mod_p(m, k, p, threads);
        r = mul_mod(r, (int64_t)n % p, p);
        free(m);
    } else {
        int64_t *m = (int64_t *)malloc((size_t)n * n * sizeof(int64_t));
        if (!m) return -1;
        int64_t wj = 1 % p;
        for (int row = 0; row < n; row++) {
            int64_t pw = 1 % p;
            for (int c = 0; c < n; c++) {
                m[row * n + c] = pw;
                pw = mul_mod(pw, wj, p);
            }
            wj = mul_mod(wj, w, p);
        }
        r = or_ryser_mod_p(m, n, p, threads);
        free(m);
    }
    return r;
}

/* Binary permanent mod an odd prime p > n (caller validates primality). */
int64_t or_binary_mod_p(const uint8_t *a, int n, int64_t p, int threads) {
    if (n < 0 || n >= 64 || p <= 2 || p <= n) return -1;
    if (n == 0) return 1 % p;
    int64_t *m = (int64_t *)malloc((size_t)n * n * sizeof(int64_t));
    if (!m) return -1;
    for (int i = 0; i < n * n; i++) {
        if (a[i] > 1) { free(m); return -1; }
        m[i] = a[i];
    }
    int64_t r = n == 1 ? m[0] : or_glynn_mod_p(m, n, p, threads);
    free(m);
    return r;
}

/* FP64 Glynn over states [lo, hi) with a Kahan-compensated sum; also sums
 * |terms| (the scale against which relative error is stated). */
static void glynn_f64_block(const double *a, int n, uint64_t lo, uint64_t hi,
                            double *sum_out, double *abs_out) {
    double rs[64];
    for (int r = 0; r < n; r++) {
        double s = 0.0;
        for (int c = 0; c < n; c++) s += a[r * n + c];
        rs[r] = s;
    }
    uint64_t g = lo ^ (lo >> 1);
    for (int c = 0; c < n - 1; c++)
        if ((g >> c) & 1)
            for (int r = 0; r < n; r++) rs[r] -= 2.0 * a[r * n + c];
    int sign = (lo & 1) ? -1 : 1;
    double sum = 0.0, comp = 0.0, asum = 0.0;
    for (uint64_t s = lo; s < hi; s++) {
        if (s != lo) {
            int c = __builtin_ctzll(s);
            uint64_t gs = s ^ (s >> 1);
            if ((gs >> c) & 1)
                for (int r = 0; r < n; r++) rs[r] -= 2.0 * a[r * n + c];
            else
                for (int r = 0; r < n; r++) rs[r] += 2.0 * a[r * n + c];
            sign = -sign;
        }
        double prod = rs[0];
        for (int r = 1; r < n; r++) prod *= rs[r];
        double y = sign * prod - comp;
        double t = sum + y;
        comp = (t - sum) - y;
        sum = t;
        asum += fabs(prod);
    }
    *sum_out = sum;
    *abs_out = asum;
}

/* Returns per(A) in FP64; *abs_sum = 2^(1-n) * sum |terms|. */
double or_glynn_f64(const double *a, int n, int threads, double *abs_sum) {
    if (n <= 0) { if (abs_sum) *abs_sum = 1.0; return 1.0; }
    if (n == 1) { if (abs_sum) *abs_sum = fabs(a[0]); return a[0]; }
    uint64_t states = 1ULL << (n - 1);
    double total = 0.0, comp = 0.0, atot = 0.0;
    int nt = threads > 1 ? threads : 1;
    if (n <= 12) nt = 1;
    double *parts = (double *)calloc((size_t)nt * 2, sizeof(double));
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int t = 0; t < nt; t++) {
        uint64_t blk = (states + (uint64_t)nt - 1) / (uint64_t)nt;
        uint64_t lo = (uint64_t)t * blk, hi = lo + blk;
        if (hi > states) hi = states;
        if (lo < hi) glynn_f64_block(a, n, lo, hi, &parts[2 * t], &parts[2 * t + 1]);
    }
    for (int t = 0; t < nt; t++) {
        double y = parts[2 * t] - comp;
        double s = total + y;
        comp = (s - total) - y;
        total = s;
        atot += parts[2 * t + 1];
    }
    free(parts);
    if (abs_sum) *abs_sum = ldexp(atot, -(n - 1));
    return ldexp(total, -(n - 1));
}

/* Complex Glynn in FP64 with a Kahan-compensated sum (serial):
 * perm_parallel_cuda.cu:68-209 with IS_COMPLEX. */
void or_glynn_c64(const double *are, const double *aim, int n, double *out_re,
                  double *out_im, double *abs_sum) {
    if (n <= 0) { *out_re = 1.0; *out_im = 0.0; if (abs_sum) *abs_sum = 1.0; return; }
    if (n == 1) { *out_re = are[0]; *out_im = aim[0]; if (abs_sum) *abs_sum = hypot(are[0], aim[0]); return; }
    double rr[64], ri[64];
    for (int r = 0; r < n; r++) {
        double sr = 0, si = 0;
        for (int c = 0; c < n; c++) { sr += are[r * n + c]; si += aim[r * n + c]; }
        rr[r] = sr; ri[r] = si;
    }
    double sr = 0, cr = 0, si = 0, ci = 0, as = 0;
    int sign = 1;
    uint64_t states = 1ULL << (n - 1);
    for (uint64_t s = 0; s < states; s++) {
        if (s) {
            int c = __builtin_ctzll(s);
            uint64_t gs = s ^ (s >> 1);
            double f = ((gs >> c) & 1) ? -2.0 : 2.0;
            for (int r = 0; r < n; r++) { rr[r] += f * are[r * n + c]; ri[r] += f * aim[r * n + c]; }
            sign = -sign;
        }
        double pr = rr[0], pi = ri[0];
        for (int r = 1; r < n; r++) {
            double nr = pr * rr[r] - pi * ri[r];
            pi = pr * ri[r] + pi * rr[r];
            pr = nr;
        }
        double y = sign * pr - cr, t = sr + y; cr = (t - sr) - y; sr = t;
        y = sign * pi - ci; t = si + y; ci = (t - si) - y; si = t;
        as += hypot(pr, pi);
    }
    *out_re = ldexp(sr, -(n - 1));
    *out_im = ldexp(si, -(n - 1));
    if (abs_sum) *abs_sum = ldexp(as, -(n - 1));
}

/* Gradient by minors: grad[i*n+j] = per(A with row i and column j removed). */
void or_glynn_f64_grad(const double *a, int n, int threads, double *grad) {
    if (n <= 0) return;
    if (n == 1) { grad[0] = 1.0; return; }
    int k = n - 1;
#pragma omp parallel for num_threads(threads > 1 ? threads : 1) schedule(dynamic)
    for (int ij = 0; ij < n * n; ij++) {
        int i = ij / n, j = ij % n;
        double minor[64 * 64];
        int q = 0;
        for (int r = 0; r < n; r++) {
            if (r == i) continue;
            for (int c = 0; c < n; c++) {
                if (c == j) continue;
                minor[q++] = a[r * n + c];
            }
        }
        double dummy;
        grad[ij] = or_glynn_f64(minor, k, 1, &dummy);
    }
}

/* Coefficients of per(C + x L) mod odd m (1 < m < 2^63), out[0..n] ascending
 * degree: 2^(1-n) sum over the 2^(n-1) fixed-sign Gray states of
 * (prod d) prod_i (c_i(d) + x l_i(d)), with c_i, l_i the signed row sums of
 * C and L (perm_polynomial.py:268-329).  Contiguous Gray blocks per thread
 * with closed-form block starts, as or_glynn_mod_p. */
static void affine_block(const int64_t *c, const int64_t *l, int n, int64_t p,
                         uint64_t lo, uint64_t hi, int64_t *acc) {
    int64_t cs[64], ls[64], poly[65], next[65];
    const uint64_t g0 = lo ^ (lo >> 1);
    for (int i = 0; i < n; i++) {
        int64_t a = 0, b = 0;
        for (int j = 0; j < n; j++) {
            int neg = j < n - 1 && ((g0 >> j) & 1);
            a = neg ? sub_mod(a, c[i * n + j], p) : add_mod(a, c[i * n + j], p);
            b = neg ? sub_mod(b, l[i * n + j], p) : add_mod(b, l[i * n + j], p);
        }
        cs[i] = a;
        ls[i] = b;
    }
    int sign_neg = __builtin_popcountll(g0) & 1;
    uint64_t g = g0;
    for (uint64_t s = lo; s < hi; s++) {
        if (s != lo) {
            const int j = __builtin_ctzll(s);
            const int sub = !((g >> j) & 1);     /* sign of column j flips to - */
            g ^= 1ull << j;
            for (int i = 0; i < n; i++) {
                const int64_t dc = add_mod(c[i * n + j], c[i * n + j], p);
                const int64_t dl = add_mod(l[i * n + j], l[i * n + j], p);
                cs[i] = sub ? sub_mod(cs[i], dc, p) : add_mod(cs[i], dc, p);
                ls[i] = sub ? sub_mod(ls[i], dl, p) : add_mod(ls[i], dl, p);
            }
            sign_neg ^= 1;
        }
        int deg = 0;
        poly[0] = 1 % p;
        for (int i = 0; i < n; i++) {
            next[0] = mul_mod(poly[0], cs[i], p);
            for (int k = 1; k <= deg; k++)
                next[k] = add_mod(mul_mod(poly[k], cs[i], p), mul_mod(poly[k - 1], ls[i], p), p);
            next[deg + 1] = mul_mod(poly[deg], ls[i], p);
            deg++;
            memcpy(poly, next, (size_t)(deg + 1) * sizeof(int64_t));
        }
        for (int k = 0; k <= n; k++)
            acc[k] = sign_neg ? sub_mod(acc[k], poly[k], p) : add_mod(acc[k], poly[k], p);
    }
}

/* Sum over Gray-ordered subsets [lo, hi) of (-1)^|S| prod_i sum_{j in S} a_ij
 * over F_3, as a count mod 3 (entries already reduced to {0,1,2}); the full
 * range times (-1)^n is per(A) mod 3.  Row sums are two bit words
 * (magnitude, sign) updated per column toggle. */
int or_mod3_range(const int64_t *A, int n, uint64_t lo, uint64_t hi, int threads) {
    if (n < 1 || n >= 64 || lo >= hi) return 0;
    uint64_t cm[64], cs[64];
    for (int j = 0; j < n; j++) {
        cm[j] = cs[j] = 0;
        for (int i = 0; i < n; i++) {
            const int v = (int)norm_mod(A[i * n + j], 3);
            if (v) cm[j] |= 1ull << i;
            if (v == 2) cs[j] |= 1ull << i;
        }
    }
    const uint64_t mask = n == 64 ? ~0ull : ((1ull << n) - 1);
    const uint64_t span = hi - lo;
    int nt = threads > 0 ? threads : 1;
    if ((uint64_t)nt > span) nt = (int)span;
    uint64_t total = 0;
#pragma omp parallel for num_threads(nt) schedule(static) reduction(+ : total)
    for (int t = 0; t < nt; t++) {
        const uint64_t b0 = lo + span / nt * t + ((uint64_t)t < span % nt ? t : span % nt);
        const uint64_t b1 = b0 + span / nt + ((uint64_t)t < span % nt ? 1 : 0);
        uint64_t m = 0, s = 0, cnt = 0;
        const uint64_t g0 = b0 ^ (b0 >> 1);
        for (int j = 0; j < n; j++)
            if ((g0 >> j) & 1) {
                const uint64_t u = m ^ s ^ cs[j], mo = (cm[j] & u) | (m ^ cm[j]);
                s = (cm[j] & u) ^ s;
                m = mo;
            }
        for (uint64_t i = b0; i < b1; i++) {
            if (i != b0) {
                const int j = __builtin_ctzll(i);
                if (((i >> (j + 1)) & 1) == 0) {          /* column j enters S */
                    const uint64_t u = m ^ s ^ cs[j], mo = (cm[j] & u) | (m ^ cm[j]);
                    s = (cm[j] & u) ^ s;
                    m = mo;
                } else {                                  /* column j leaves S */
                    const uint64_t u = s ^ cs[j], mo = (m & u) | (m ^ cm[j]);
                    s = (m & u) ^ (cm[j] ^ cs[j]);
                    m = mo;
                }
            }
            if ((m & mask) == mask)
                cnt += 1 + ((__builtin_popcountll(s & mask) ^ (int)(i & 1)) & 1);
        }
        total += cnt % 3;
    }
    return (int)(total % 3);
}

int or_permanent_mod3(const int64_t *A, int n, int threads) {
    if (n == 0) return 1;
    if (n == 1) return (int)norm_mod(A[0], 3);
    const int t = or_mod3_range(A, n, 0, 1ull << n, threads);
    return (n & 1) ? (3 - t) % 3 : t;
}

/* Unscaled partial coefficient sums over Gray states [lo, hi) (the CPU
 * baseline sample of or_affine_mod_p), split over `threads` OpenMP threads. */
int or_affine_range_mod_p(const int64_t *C, const int64_t *L, int n, int64_t p, uint64_t lo,
                          uint64_t hi, int threads, int64_t *out) {
    if (n < 2 || n >= 64 || p < 3 || !(p & 1) || lo >= hi) return -1;
    int64_t *c = (int64_t *)malloc(sizeof(int64_t) * (size_t)n * n * 2);
    if (!c) return -1;
    int64_t *l = c + (size_t)n * n;
    for (int i = 0; i < n * n; i++) {
        c[i] = norm_mod(C[i], p);
        l[i] = norm_mod(L[i], p);
    }
    const uint64_t span = hi - lo;
    int nt = threads > 0 ? threads : 1;
    if ((uint64_t)nt > span) nt = (int)span;
    int64_t *accs = (int64_t *)calloc((size_t)nt * 65, sizeof(int64_t));
    if (!accs) { free(c); return -1; }
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int t = 0; t < nt; t++) {
        const uint64_t b0 = lo + span / nt * t + ((uint64_t)t < span % nt ? t : span % nt);
        const uint64_t len = span / nt + ((uint64_t)t < span % nt ? 1 : 0);
        affine_block(c, l, n, p, b0, b0 + len, accs + (size_t)t * 65);
    }
    for (int k = 0; k <= n; k++) {
        int64_t s = 0;
        for (int t = 0; t < nt; t++) s = add_mod(s, accs[(size_t)t * 65 + k], p);
        out[k] = s;
    }
    free(accs);
    free(c);
    return 0;
}

int or_affine_mod_p(const int64_t *C, const int64_t *L, int n, int64_t p, int threads,
                    int64_t *out) {
    if (n < 0 || n >= 64 || p < 3 || !(p & 1)) return -1;
    if (n == 0) { out[0] = 1 % p; return 0; }
    int64_t *c = (int64_t *)malloc(sizeof(int64_t) * (size_t)n * n * 2);
    if (!c) return -1;
    int64_t *l = c + (size_t)n * n;
    for (int i = 0; i < n * n; i++) {
        c[i] = norm_mod(C[i], p);
        l[i] = norm_mod(L[i], p);
    }
    if (n == 1) {
        out[0] = c[0];
        out[1] = l[0];
        free(c);
        return 0;
    }
    const uint64_t states = 1ull << (n - 1);
    int nt = threads > 0 ? threads : 1;
    if ((uint64_t)nt > states) nt = (int)states;
    int64_t *accs = (int64_t *)calloc((size_t)nt * 65, sizeof(int64_t));
    if (!accs) { free(c); return -1; }
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int t = 0; t < nt; t++) {
        const uint64_t lo = states / nt * t + ((uint64_t)t < states % nt ? t : states % nt);
        const uint64_t len = states / nt + ((uint64_t)t < states % nt ? 1 : 0);
        affine_block(c, l, n, p, lo, lo + len, accs + (size_t)t * 65);
    }
    const int64_t inv2 = (p >> 1) + 1;
    const int64_t scale = pow_mod(inv2, (uint64_t)(n - 1), p);
    for (int k = 0; k <= n; k++) {
        int64_t s = 0;
        for (int t = 0; t < nt; t++) s = add_mod(s, accs[(size_t)t * 65 + k], p);
        out[k] = mul_mod(s, scale, p);
    }
    free(accs);
    free(c);
    return 0;
}
