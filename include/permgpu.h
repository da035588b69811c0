/*
 * permgpu — C ABI of the GB300 (sm_103a) exact-permanent engines.
 *
 * Plain C types only: host pointers in, host pointers out (the *_dev entry
 * points take device pointers and a cudaStream_t passed as void*).  Every
 * entry point returns a pg_status; pg_last_error() gives a message for the
 * calling thread.  The library keeps no __constant__ state, so calls from
 * several host threads are safe (each call synchronises its own stream).
 *
 * Each entry point names the reference interface it replaces
 * (rivin-perm, file:line).
 */
#ifndef PERMGPU_H
#define PERMGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PG_OK = 0,
    PG_EINVAL = 1,     /* malformed argument (null pointer, bad shape, entry) */
    PG_ERANGE = 2,     /* order / modulus / limb count outside the contract */
    PG_ECUDA = 3,      /* CUDA runtime error (message in pg_last_error) */
    PG_ENOMEM = 4,     /* device or host allocation failed */
    PG_EABORT = 5,     /* pg_abort() was called while the launch ran */
    PG_ENODEV = 6,     /* no CUDA device visible */
    PG_EOVERFLOW = 7,  /* exact engine: bound exceeds its fixed-width range */
    PG_EINTERNAL = 8   /* self-check failed (e.g. Glynn sum not divisible by
                          2^(n-1)); the result was not written */
} pg_status;

/* Library version (major*10000 + minor*100 + patch). */
int pg_version(void);

/* 1 if a CUDA device is usable; replaces cuda_runtime_available()
 * (perm_modp_cuda.cu:731). */
int pg_cuda_runtime_available(void);

/* Message describing the last failure on the calling host thread. */
const char *pg_last_error(void);

/* SM count and compute capability of the current device. */
int pg_device_info(int *sm_count, int *cc_major, int *cc_minor);

/* Ask running launches to stop at their next poll; they return PG_EABORT.
 * A kernel thread reads the abort word once per 2^16 states (per chunk
 * for longer chunks) from its second period on, so launches whose threads
 * walk fewer states complete.  pg_clear_abort() re-arms the library. */
void pg_abort(void);
void pg_clear_abort(void);

/*
 * Residue engine: out[t] = per(A) mod moduli[t] for t < k.
 *   A       row-major n x n signed 64-bit entries (any values; reduced mod
 *           each modulus on the host exactly as perm_c_omp.c:911 does)
 *   n       0 <= n < 64
 *   moduli  1 <= m < 2^63, any parity (odd m < 2^31 run the 32-bit
 *           Montgomery Glynn kernel; odd m < 2^32 its fully reduced wide
 *           form; larger odd m the 64-bit one; even m split as 2^e * odd
 *           with a wrap-around Ryser kernel for 2^e)
 * Replaces perm_c_ext.permanent_mod_p / ryser_permanent_mod_p
 * (perm_c_omp.c:858-937, dispatch :846-854) and permanent_modp_cuda
 * (perm_modp_cuda.cu:740-868).  All odd moduli below 2^31 share one launch.
 */
int pg_residues(const int64_t *A, int n, const uint64_t *moduli, int k,
                uint64_t *out);

/*
 * Sharded residues: out[t] = the unscaled Glynn sum over Gray states
 * [state_lo, state_hi) (both even, lo < hi <= 2^(n-1)) mod moduli[t], i.e.
 * without the 2^(1-n) factor, for odd moduli 3 <= m < 2^32 and 2 <= n < 64.
 * Summing the values of a partition of [0, 2^(n-1)) mod m and multiplying
 * by 2^(1-n) gives per(A) mod m (permgpu.shard.combine_residues), so ranks
 * can split one modulus's traversal.  The reference's OpenMP loop splits
 * the same Gray walk across threads (perm_c_omp.c:556-639).
 */
int pg_residues_partial(const int64_t *A, int n, uint64_t state_lo, uint64_t state_hi,
                        const uint64_t *moduli, int k, uint64_t *out);

/*
 * Schur residues: out[t] = perm(S_n) mod primes[t] with S_n[j][c] =
 * omegas[t]^(j*c).  For odd n, odd p and omega^n == 1 this evaluates
 * n * per(minor) with the (n-1)x(n-1) minor omega^((r+1)(c+1)); otherwise
 * the full matrix.  Replaces perm_c_ext.schur_permanent_mod_p
 * (perm_c_omp.c:942-1060) and schur_permanent_modp_cuda
 * (perm_modp_cuda.cu:1266-1348).  0 <= n < 64, 1 <= p < 2^63.
 */
int pg_schur_residues(int n, const uint64_t *primes, const uint64_t *omegas,
                      int k, uint64_t *out);

/*
 * Schur residues with an explicit evaluation method.  PG_SCHUR_AUTO is
 * pg_schur_residues: the necklace quotient where it applies and n >= 37,
 * else the Glynn cofactor minor, else the full matrix.  PG_SCHUR_GLYNN
 * forces the cofactor minor (2^(n-2) Glynn states).  PG_SCHUR_NECKLACE
 * requires the necklace preconditions (odd prime n < 64, odd modulus
 * < 2^30, or < 2^32 for n = 37, 41, 43, 47, 53, omega^n == 1) for every
 * modulus and returns PG_ERANGE otherwise: the
 * (n-1)x(n-1) cofactor minor is circulant in primitive-root order and its
 * 2^(n-1) Glynn sign words collapse to rotation+complement orbits, about
 * 2^(n-1)/(2(n-1)) terms.  Replaces the necklace branch of
 * perm_c_ext.schur_permanent_mod_p (perm_c_omp.c:977-1012; enumeration
 * :89-153, minor :193-226, evaluation :228-305, :416-507) and
 * schur_necklace_modp_cuda (perm_modp_cuda.cu:957-1090, kernel :524-705).
 */
enum pg_schur_method { PG_SCHUR_AUTO = 0, PG_SCHUR_GLYNN = 1, PG_SCHUR_NECKLACE = 2 };
int pg_schur_residues_method(int n, const uint64_t *primes, const uint64_t *omegas,
                             int k, int method, uint64_t *out);

/*
 * Necklace quotient statistics for an odd prime order 3 <= n < 64:
 * number of orbit representatives and the number of sign words they cover
 * (2^(n-1) when the quotient is complete).  Host only, no GPU needed.
 * Replaces perm_c_ext.schur_necklace_orbit_stats (perm_c_omp.c:1062-1082).
 */
int pg_necklace_orbit_stats(int n, uint64_t *representatives, uint64_t *words);

/*
 * Affine-polynomial residues: out[t*(n+1) + d] = coefficient of x^d in
 * per(C + x L) mod moduli[t], for row-major n x n signed 64-bit C and L,
 * 0 <= n <= 63 and odd moduli 3 <= m < 2^30 (they need not be prime).  All
 * moduli run in one launch.  Replaces perm_polynomial_ext.affine_permanent_mod
 * (perm_polynomial_omp.c:1207-1360, engine :434-486, :612-779); the
 * principal-permanent polynomial per(I + x A) and the rook polynomials
 * per(J + x A) (perm_polynomial.py:1217-1287, :1288-1411, :1512-1606) are
 * this entry with C = I or C = J.
 */
int pg_affine_residues(const int64_t *C, const int64_t *L, int n,
                       const uint64_t *moduli, int k, uint64_t *out);

/*
 * pg_affine_residues restricted to the Gray states [state_lo, state_hi) of
 * the walk (2 <= n <= 63): out[t*(n+1) + d] = coefficient of x^d of the
 * unscaled Glynn sum over those states, sum_g (-1)^g prod_i (c_i(g) +
 * x l_i(g)) mod moduli[t] (NOT multiplied by 2^(1-n)).  Windows of a
 * partition of [0, 2^(n-1)) add up to 2^(n-1) per(C + x L); they split one
 * polynomial across devices the way the reference's native engine splits
 * the walk across threads (perm_polynomial_omp.c:612-636).  The window
 * interface has no reference counterpart.
 */
int pg_affine_residues_partial(const int64_t *C, const int64_t *L, int n,
                               uint64_t state_lo, uint64_t state_hi,
                               const uint64_t *moduli, int k, uint64_t *out);

/*
 * Permanent modulo 3 (*out in {0, 1, 2}) by Ryser's formula over F_3 with
 * bit-sliced row sums, 0 <= n < 64, any int64 entries.  Replaces
 * permanent_mod3_matrix (perm_mod3_cuda.cu:300-349) and the OpenMP
 * perm_mod3_omp.permanent_mod3 behind perm_mod3.permanent_mod3_fast
 * (perm_mod3.py:355-383).
 */
int pg_permanent_mod3(const int64_t *A, int n, int *out);

/*
 * The same from the F_3 column encodings: bit i of col_mags[j] is set when
 * a_ij != 0 (mod 3), bit i of col_sgns[j] when a_ij == 2 (mod 3); sign bits
 * must lie inside the magnitude bits.  Replaces permanent_mod3_cuda
 * (perm_mod3_cuda.cu:164-296), encodings as perm_mod3.encode_matrix_f3.
 */
int pg_permanent_mod3_cols(const uint64_t *col_mags, const uint64_t *col_sgns,
                           int n, int *out);

/*
 * Binary residues: out[t] = per(A) mod primes[t] for a 0/1 matrix.
 * Contract of perm_binary_ext.binary_permanent_mod_p (perm_binary_omp.c:
 * 386-519) and binary_permanent_modp_cuda (perm_binary_cuda.cu:471-482):
 * entries must be 0 or 1, 0 <= n < 64, each prime odd, prime and > n.
 */
int pg_binary_residues(const uint8_t *A, int n, const uint64_t *primes, int k,
                       uint64_t *out);

/*
 * Exact engine: per(A) as a two's-complement little-endian integer of
 * `limbs` 32-bit words.  Row sums are kept as exact int32 and every Glynn
 * term is formed as an exact multi-word product, so no CRT is needed.
 * Returns PG_EOVERFLOW (nothing written) when the row-sum bound
 * prod_i sum_j |a_ij| does not fit the compiled widths; callers then use
 * pg_residues + CRT.  Replaces the whole residue loop of
 * perm.matrix_permanent(A, method="generic") (perm.py:1076-1212).
 */
int pg_exact_permanent(const int64_t *A, int n, uint32_t *out, int limbs);

/* 1 if pg_exact_permanent accepts this matrix (bound fits), else 0. */
int pg_exact_supported(const int64_t *A, int n);

/*
 * Sharded exact evaluation: the unscaled Glynn sum over Gray states
 * [state_lo, state_hi) (multiples of 4) as *nwords 64-bit words, word w of
 * weight 2^(32 w), the last word signed.  Summing the words of a partition
 * of [0, 2^(n-1)) over ranks/hosts and dividing by 2^(n-1) gives per(A).
 * Same matrix contract as pg_exact_permanent; mirrors the contiguous
 * Gray-block split of perm_c_omp.c:565-603 across devices instead of
 * threads.
 */
int pg_exact_partial(const int64_t *A, int n, uint64_t state_lo,
                     uint64_t state_hi, int64_t *words, int max_words,
                     int *nwords);

/*
 * Reusable exact plan: the host work of pg_exact_permanent (grouping, column
 * tables, launch shape) done once and the tables kept resident in device
 * memory, so repeated evaluations pay only the launch.  `stream` may be NULL
 * (the plan's own stream) or a cudaStream_t.  launch is asynchronous;
 * result copies the per-word sums back, synchronises `stream` and writes
 * per(A) as in pg_exact_permanent.  Same contract as pg_exact_permanent
 * (perm.py:1076-1212 whole-call replacement), split for device-resident
 * timing and for callers that re-evaluate one matrix.
 */
typedef struct pg_exact_plan pg_exact_plan;
int pg_exact_plan_create(const int64_t *A, int n, pg_exact_plan **plan);
int pg_exact_plan_launch(pg_exact_plan *plan, void *stream);
int pg_exact_plan_result(pg_exact_plan *plan, void *stream, uint32_t *out,
                         int limbs);
/* group size, product words, Gray states, and per-state counts of 32-bit
 * row-group multiplies and 32x32->64 word products of the launch (the
 * roofline's work unit; the float-row form runs two of every three group
 * multiplies as exact FP32 multiplies). */
int pg_exact_plan_info(const pg_exact_plan *plan, int *group, int *words,
                       uint64_t *states, uint64_t *imul_per_state,
                       uint64_t *imad_wide_per_state);
/* Float rows per row group of the plan (0: integer form); with FR > 0 each
 * group of G rows runs FR - 1 of its G - 1 multiplies on the FP32 pipe and
 * G - FR as 32-bit IMULs.  Splits pg_exact_plan_info's multiply count by
 * pipe for the roofline (no reference counterpart). */
int pg_exact_plan_float_rows(const pg_exact_plan *plan);
/* Offset planes of the plan's 0/1 kernel (0/1 matrices of orders 24..48
 * whose sampled share of states without a zero row is at most 1/4 run a
 * bit-sliced walk over the even-degree rows' offsets from half their degree,
 * modulo 2^K, with exact evaluation of the surviving states); 0 when the
 * general exact kernel runs.  The binary
 * counterpart of rivin-perm's binary_glynn_mont32 / binary_glynn_ratio_kernel
 * (perm_binary_omp.c:236-347, perm_binary_cuda.cu:111-205), which it
 * replaces on the binary_permanent path with an exact result. */
int pg_exact_plan_bit_planes(const pg_exact_plan *plan);
void pg_exact_plan_destroy(pg_exact_plan *plan);

/*
 * Batched exact engine: per(A_m) for `count` matrices of uneven order in one
 * persistent, work-stealing launch captured in a CUDA graph.  Matrix m is
 * the row-major n_m x n_m block at A + offsets[m] (n_m = orders[m]).
 * out receives `limbs` two's-complement words per matrix.  Orders 2..32
 * whose rows group into products < 2^31 run inside the batched kernel; any
 * other matrix is evaluated by pg_exact_permanent when results are
 * collected (PG_EOVERFLOW if even that engine cannot take it).  Replaces a
 * per-matrix loop over perm.matrix_permanent(A, method="generic")
 * (perm.py:1076-1212); there is no batched entry point in the reference.
 * pg_batch_tune fields <= 0 select the defaults (13, 6, 2).
 */
typedef struct {
    int lane_log_states;   /* log2 Gray states per lane per task */
    int chunk_log_len;     /* log2 states per aligned chunk */
    int blocks_per_sm;     /* resident blocks of 256 threads per SM */
} pg_batch_tune;
typedef struct pg_batch_plan pg_batch_plan;
int pg_batch_plan_create(const int64_t *A, const int64_t *offsets,
                         const int32_t *orders, int count,
                         const pg_batch_tune *tune, pg_batch_plan **plan);
int pg_batch_plan_launch(pg_batch_plan *plan, void *stream);
int pg_batch_plan_result(pg_batch_plan *plan, void *stream, uint32_t *out,
                         int limbs);
int pg_batch_plan_info(const pg_batch_plan *plan, uint32_t *tasks,
                       int *blocks, uint64_t *kernel_states, int *external);
void pg_batch_plan_destroy(pg_batch_plan *plan);
/*
 * Residues of many matrices, each modulo its own moduli:
 *   out[moduli_offsets[m] + t] = per(A_m) mod moduli[moduli_offsets[m] + t]
 * for t < moduli_offsets[m+1] - moduli_offsets[m]; A_m is the row-major
 * orders[m]^2 block at A + offsets[m].  Matrices the exact engine accepts
 * run in one batched exact launch (results reduced on the host); the others
 * take pg_residues with all their moduli in one launch.  Replaces the
 * per-matrix, per-prime loop over permanent_mod_p (perm.py:1172-1197).
 */
int pg_batch_residues(const int64_t *A, const int64_t *offsets,
                      const int32_t *orders, int count,
                      const uint64_t *moduli, const int32_t *moduli_offsets,
                      uint64_t *out);
int pg_batch_exact(const int64_t *A, const int64_t *offsets,
                   const int32_t *orders, int count, uint32_t *out, int limbs);

/*
 * FP64 Glynn permanent and gradient for a batch of real matrices, device
 * pointers (torch tensors) on `stream` (NULL: the library's stream):
 *   per[b]          = per(A_b)                       (A: [batch][n][n] f64)
 *   grad[b][i][j]   = d per / d a_ij = per(A_b without row i, column j)
 *   abs_sum[b]      = 2^(1-n) sum |terms|  (error scale of per[b])
 *   grad_abs[b][i]  = 2^(1-n) sum |prod_{l != i} s_l|  (scale of row i)
 * grad / abs_sum / grad_abs may be NULL (grad NULL: forward only).
 * 2 <= n <= 63; the gradient for n <= 32 (orders 33..63 run forward only,
 * two rows per lane, and return PG_ERANGE when grad or grad_abs is given).
 * Replaces permanent_parallel_real (perm_parallel_cuda.cu:343-414, forward
 * only, one matrix, n <= 63); the gradient has no reference counterpart.
 * Synchronises `stream` before returning.
 */
int pg_glynn_f64_dev(const double *A, int batch, int n, double *per,
                     double *grad, double *abs_sum, double *grad_abs,
                     void *stream);

/*
 * pg_glynn_f64_dev with host pointers: A [batch][n][n] f64 in, per[batch],
 * grad [batch][n][n] (NULL: forward only) and abs_sum[batch] (nullable)
 * out; 0 <= n <= 63 (gradient: n <= 32).  Device buffers for the call are allocated and freed
 * inside, so plain ctypes callers need no device memory of their own.
 * Replaces permanent_parallel_real (perm_parallel_cuda.cu:343-414) for a
 * whole batch, with the gradient.
 */
int pg_glynn_f64_fwd_bwd(const double *A, int batch, int n, double *per,
                         double *grad, double *abs_sum);

/*
 * Complex FP64 Glynn permanent (forward) for a batch of complex matrices
 * given as separate real and imaginary planes (device pointers, [batch][n]
 * [n] each); per_re/per_im receive per(A_b), abs_sum (nullable) the error
 * scale 2^(1-n) sum |terms|.  2 <= n <= 63.  Replaces
 * permanent_parallel_complex (perm_parallel_cuda.cu:416-498).
 */
int pg_glynn_c64_dev(const double *Are, const double *Aim, int batch, int n,
                     double *per_re, double *per_im, double *abs_sum,
                     void *stream);

/*
 * pg_glynn_c64_dev with host pointers: real and imaginary planes
 * [batch][n][n] in, per_re/per_im[batch] and abs_sum[batch] (nullable) out;
 * 0 <= n <= 63.  Device buffers for the call are allocated and freed
 * inside.  Replaces permanent_parallel_complex (perm_parallel_cuda.cu:
 * 416-498) for a whole batch.
 */
int pg_glynn_c64(const double *Are, const double *Aim, int batch, int n,
                 double *per_re, double *per_im, double *abs_sum);

/*
 * FP64 Glynn sum over a Gray window of one real (Aim NULL) or complex
 * matrix, host pointers: sum_re/sum_im = sum over states g in [lo, hi) of
 * (-1)^g prod_i s_i(g), with s_i(g) = sum_j d_j(g) a_ij and the last
 * column's sign fixed, NOT divided by 2^(n-1); abs_sum (nullable) = the sum
 * of |terms| over the window (its error scale).  2 <= n <= 63,
 * lo <= hi <= 2^(n-1).  Windows split one FP64 permanent across devices
 * (per(A) = 2^(1-n) times the sum of the window sums) the way rivin-perm's
 * permanent_glynn_kernel splits the walk across threads
 * (perm_parallel_cuda.cu:68-209); the window interface itself has no
 * reference counterpart.
 */
int pg_glynn_window(const double *Are, const double *Aim, int n, uint64_t lo,
                    uint64_t hi, double *sum_re, double *sum_im, double *abs_sum);

/*
 * pg_exact_permanent for callers that cannot allocate memory (no
 * counterpart in the reference).  Plug-ins whose host process owns every
 * device allocation through its own pool, and services that reserve a fixed
 * device-memory budget at start-up and must not grow it, cannot call
 * cudaMalloc; this entry point allocates nothing (no device, pinned or host
 * heap memory, no streams).  Its scratch is a fixed 32 KiB __device__ array
 * inside the library, present on every GPU that loads it until exit; orders
 * 2..48 fit, anything larger returns PG_ERANGE, and so does a limb count too
 * small for the permanent's bound.  It runs the exact kernel's integer-row
 * form only (slower than pg_exact_permanent at orders 24..32).  The caller
 * passes the host matrix and the host output words; `stream` may be NULL
 * (legacy default stream) and is synchronised before the call returns.
 * All calls share the scratch: calls that overlap on the GPU race and must
 * be serialised by the caller.  The first call on each device looks up the
 * scratch address (cudaGetSymbolAddress) and keeps it for the process's
 * life; calls after cudaDeviceReset are not supported.  pg_abort() stops it only once
 * the process's abort word exists (any allocating entry point, pg_abort or
 * pg_clear_abort creates it; this entry point does not).
 */
int pg_exact_permanent_noalloc(const int64_t *A, int n, uint32_t *out,
                               int limbs, void *stream);

/*
 * Pipe throughput probe (roofline denominator; a measurement utility with
 * no reference counterpart): variant 0 mad.lo.u32, 1 mad.wide.u32 (64-bit
 * addend), 2 mad.hi.u32, 3 add.u32, 4 mul.wide.u32 (no addend), 5
 * fma.rn.f32, 6 fma.rn.f64; writes thread-instructions per second for the
 * whole GPU.
 */
int pg_probe_int_throughput(int variant, int iters, double *ops_per_second);

#ifdef __cplusplus
}
#endif

#endif /* PERMGPU_H */
