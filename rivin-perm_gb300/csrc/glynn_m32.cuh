// Multi-prime Glynn residue kernel, 32-bit Montgomery arithmetic.
//
// per(A) = 2^(1-n) * sum_{d in {+-1}^(n-1) x {+1}} (prod_j d_j) prod_i s_i(d),
// s_i(d) = sum_j d_j a_ij (rivin-perm perm_c_omp.c:510-639).  The 2^(n-1)
// states are walked in Gray order in aligned chunks (one chunk per thread per
// grid-stride step).  Alignment means the column toggled at local step i is
// ctz(i) for every chunk, so the whole warp reads one column: the column
// table lives in shared memory and every read is a broadcast.
//
// Arithmetic: odd modulus p < 2^31, row sums kept in [0, p) and updated with
// one IADD3 + one VIADDMNMX (min(s+d-p, s+d)), the row product is a chain of
// N-1 Montgomery reductions (mul.wide, mul.lo, mad.wide) with the running
// product in [0, 2p) and no conditional subtraction.  The chain multiplies in
// R^-(N-1), R = 2^32, which the host removes together with 2^(1-n).
//
// One block handles one modulus (blockIdx.y); each block reduces its
// threads' residues and adds one 64-bit word to acc[blockIdx.y].
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#ifndef M32_LOGU
#define M32_LOGU 1
#endif

namespace pg {

struct M32Args {
    const uint32_t *tabs;      // [k][N-1][2][NP] (d - p) mod 2^32, dir 0 add / 1 sub
    const uint32_t *init;      // [k][NP] row sums of the all-plus state, in [0, p)
    const uint32_t *moduli;    // [k]
    const uint32_t *pinvs;     // [k]  -p^-1 mod 2^32
    unsigned long long *acc;   // [k]  zeroed by the host
    int *status;               // set to 1 when the abort flag stopped the launch
    volatile const int *abort_flag;
    uint64_t chunks;           // chunks per modulus: [chunk0, chunk0 + chunks)
    int log_len;               // chunk length 2^log_len, LOGU <= log_len <= 30
    uint64_t chunk0;           // first chunk (0 for a whole traversal)
};

__device__ __forceinline__ uint32_t m32_redc_mul(uint32_t a, uint32_t b,
                                                 uint32_t p, uint32_t pinv) {
    // a < 2p, b < p, p < 2^31: a*b + m*p < 2^64 and the result is < 2p.
    uint64_t t = (uint64_t)a * b;
    uint32_t m = (uint32_t)t * pinv;
    uint64_t u = (uint64_t)m * p + t;
    return (uint32_t)(u >> 32);
}

// Wide moduli 2^31 <= p < 2^32 (the 2^32 - c primes): values are kept fully
// reduced in [0, p) and intermediate sums take 33 bits.
// (a + b) mod p for a, b < p < 2^32
__device__ __forceinline__ uint32_t m32w_addmod(uint32_t a, uint32_t b, uint32_t p) {
    const uint64_t s = (uint64_t)a + b;
    return s >= p ? (uint32_t)(s - p) : (uint32_t)s;
}

// a * b * 2^-32 mod p for a, b < p < 2^32, fully reduced.  With
// m = -t p^-1 mod 2^32 the low words of t and m*p add to 0 or exactly 2^32
// (a carry iff lo(t) != 0), and (t + m*p) / 2^32 < 2p needs 33 bits.
__device__ __forceinline__ uint32_t m32w_redc_mul(uint32_t a, uint32_t b, uint32_t p,
                                                  uint32_t pinv) {
    const uint64_t t = (uint64_t)a * b;
    const uint32_t m = (uint32_t)t * pinv;
    const uint64_t mp = (uint64_t)m * p;
    const uint64_t u = (t >> 32) + (mp >> 32) + ((uint32_t)t != 0u);
    return u >= p ? (uint32_t)(u - p) : (uint32_t)u;
}

__device__ __forceinline__ constexpr int ctz_small(int r) {
    return (r & 1) ? 0 : (r & 2) ? 1 : (r & 4) ? 2 : (r & 8) ? 3 : 4;
}

__device__ __forceinline__ uint32_t m32_addmod(uint32_t s, uint32_t dm,
                                               uint32_t p) {
    // s in [0,p), dm = d - p with d in [0,p]: returns (s + d) mod p.
    return __viaddmin_u32(s, dm, s + dm + p);
}

// Resident blocks per SM requested from ptxas: enough registers for the N
// row sums plus ~40 of working set, so more warps hide the IMAD latency.
__host__ __device__ constexpr int m32_min_blocks(int N) {
    return (65536 / (256 * (N + 40))) < 1 ? 1
           : (65536 / (256 * (N + 40))) > 4 ? 4
           : (65536 / (256 * (N + 40)));
}

// W: wide moduli (2^31 <= p < 2^32).  The tables then hold the plain
// residues of +2a and -2a, sums and products stay fully reduced.
template <int N, bool W = false>
__global__ void __launch_bounds__(256, m32_min_blocks(N))
glynn_m32_kernel(M32Args a) {
    constexpr int NP = (N + 3) & ~3;
    constexpr int NCOL = N - 1;
    constexpr int LOGU = (N - 1) < M32_LOGU ? (N - 1) : M32_LOGU;
    constexpr int U = 1 << LOGU;
    extern __shared__ uint4 smem_u4[];
    uint32_t *tab = reinterpret_cast<uint32_t *>(smem_u4);

    const int k = blockIdx.y;
    {
        const uint4 *g = reinterpret_cast<const uint4 *>(
            a.tabs + (size_t)k * NCOL * 2 * NP);
        for (int i = threadIdx.x; i < NCOL * 2 * NP / 4; i += blockDim.x)
            smem_u4[i] = g[i];
    }
    __syncthreads();

    const uint32_t p = a.moduli[k];
    const uint32_t pinv = a.pinvs[k];
    const uint32_t *init = a.init + (size_t)k * NP;
    const uint32_t Q = (1u << a.log_len) >> LOGU;
    unsigned long long thread_sum = 0;
    bool aborted = false;

    // Contiguous, balanced chunk range per thread (see exact_glynn.cuh):
    // initialise once, cross chunk boundaries with an ordinary Gray step.
    const uint64_t T = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t c_begin = a.chunk0 + tid * a.chunks / T;
    const uint64_t c_end = a.chunk0 + (tid + 1) * a.chunks / T;

    uint32_t s[N];
    if (c_begin < c_end) {
        const uint64_t start = c_begin << a.log_len;
        const uint64_t gstart = start ^ (start >> 1);
#pragma unroll
        for (int i = 0; i < N; i++) s[i] = init[i];
        for (int j = 0; j < NCOL; j++) {
            if ((gstart >> j) & 1) {
                const uint32_t *col = tab + (2 * j + 1) * NP;
#pragma unroll
                for (int i = 0; i < N; i++)
                    s[i] = W ? m32w_addmod(s[i], col[i], p) : m32_addmod(s[i], col[i], p);
            }
        }
    }

    // the host-mapped abort word is read once per 2^16 states (per chunk for
    // longer chunks), from the thread's second period on: threads of a short
    // launch never read it, so thousands of warps do not queue on one
    // host-memory word before their work starts
    const uint64_t poll = a.log_len >= 16 ? 0 : (1ull << (16 - a.log_len)) - 1;
    for (uint64_t c = c_begin; c < c_end; c++) {
        if (c != c_begin && ((c - c_begin) & poll) == 0 && *a.abort_flag) { aborted = true; break; }
        // bits 0..log_len of the global state index g = c * 2^log_len + i
        const uint32_t hib = (uint32_t)(c & 1) << a.log_len;
        unsigned long long acc_e = 0, acc_o = 0;
        for (uint32_t q = 0; q < Q; q++) {
            const uint32_t g32 = (q << LOGU) | hib;
#pragma unroll
            for (int r = 0; r < U; r++) {
                bool step = true;
                int j, sub;
                if (r != 0) {
                    j = ctz_small(r);
                    if (j + 1 < LOGU) sub = ((r >> (j + 1)) & 1) == 0;
                    else sub = ((g32 >> LOGU) & 1) == 0;
                } else if (q != 0) {
                    j = __ffs(q) - 1 + LOGU;
                    sub = ((g32 >> (j + 1)) & 1) == 0;
                } else {
                    // chunk boundary (lanes may toggle different columns)
                    step = c != c_begin;
                    const int jc = __ffsll((long long)c) - 1;
                    j = a.log_len + jc;
                    sub = ((c >> (jc + 1)) & 1) == 0;
                }
                if (step) {
                    const uint4 *col =
                        reinterpret_cast<const uint4 *>(tab + (2 * j + sub) * NP);
                    const auto add = [&](uint32_t x, uint32_t d) {
                        return W ? m32w_addmod(x, d, p) : m32_addmod(x, d, p);
                    };
#pragma unroll
                    for (int v = 0; v < NP / 4; v++) {
                        const uint4 d = col[v];
                        if (4 * v + 0 < N) s[4 * v + 0] = add(s[4 * v + 0], d.x);
                        if (4 * v + 1 < N) s[4 * v + 1] = add(s[4 * v + 1], d.y);
                        if (4 * v + 2 < N) s[4 * v + 2] = add(s[4 * v + 2], d.z);
                        if (4 * v + 3 < N) s[4 * v + 3] = add(s[4 * v + 3], d.w);
                    }
                }
                // NCH independent REDC chains over interleaved rows, then a
                // combining tree; each combine first brings one side below p.
                constexpr int NCH = N >= 16 ? 4 : (N >= 4 ? 2 : 1);
                // narrow: chains below 2p, one side of each combine brought
                // below p; wide: everything fully reduced
                const auto mul = [&](uint32_t x, uint32_t y) {
                    return W ? m32w_redc_mul(x, y, p, pinv) : m32_redc_mul(x, y, p, pinv);
                };
                const auto low = [&](uint32_t x) {
                    return W ? x : __viaddmin_u32(x, 0u - p, x);
                };
                uint32_t ch[NCH];
#pragma unroll
                for (int t = 0; t < NCH; t++) ch[t] = s[t];
#pragma unroll
                for (int i = NCH; i < N; i++) ch[i % NCH] = mul(ch[i % NCH], s[i]);
                uint32_t prod;
                if (NCH == 4) {
                    const uint32_t c01 = mul(ch[0], low(ch[1]));
                    const uint32_t c23 = mul(ch[2], low(ch[3]));
                    prod = mul(c01, low(c23));
                } else if (NCH == 2) {
                    prod = mul(ch[0], low(ch[1]));
                } else {
                    prod = ch[0];
                }
                // Glynn sign (-1)^g = (-1)^r: chunks start at even states
                if (r & 1) acc_o += prod;
                else acc_e += prod;
            }
        }
        const uint32_t e = (uint32_t)(acc_e % p), o = (uint32_t)(acc_o % p);
        thread_sum += e >= o ? e - o : e + (p - o);
    }

    // block reduction of the per-thread residues (< 2^32 each after the
    // fold, so the 64-bit atomic sum over all blocks cannot overflow)
    thread_sum %= p;
    __shared__ unsigned long long red[8];
    __shared__ int any_abort;
    if (threadIdx.x == 0) any_abort = 0;
    __syncthreads();
    if (aborted) any_abort = 1;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        thread_sum += __shfl_down_sync(0xffffffffu, thread_sum, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = thread_sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        atomicAdd(a.acc + k, t);
        if (any_abort) atomicExch(a.status, 1);
    }
}

// Launch helper: grid (blocks_per_modulus, k), 256 threads, dynamic smem for
// one modulus table.  Returns cudaError_t of the launch.
template <int N, bool W = false>
cudaError_t launch_glynn_m32(const M32Args &args, int k, int blocks_per_mod,
                             cudaStream_t stream) {
    constexpr int NP = (N + 3) & ~3;
    const size_t smem = (size_t)(N - 1) * 2 * NP * sizeof(uint32_t);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(
            glynn_m32_kernel<N, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
            (int)smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid(blocks_per_mod, k);
    glynn_m32_kernel<N, W><<<grid, 256, smem, stream>>>(args);
    return cudaGetLastError();
}

template <int N, bool W = false>
int occupancy_glynn_m32() {
    constexpr int NP = (N + 3) & ~3;
    const size_t smem = (size_t)(N - 1) * 2 * NP * sizeof(uint32_t);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(glynn_m32_kernel<N, W>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, glynn_m32_kernel<N, W>, 256,
                                                      smem) != cudaSuccess)
        return 1;
    return nb < 1 ? 1 : nb;
}

// Dispatch over the compiled orders 2..63 (split across translation units).
cudaError_t launch_glynn_m32_lo(int N, const M32Args &args, int k,
                                int blocks_per_mod, cudaStream_t stream);
cudaError_t launch_glynn_m32_mid(int N, const M32Args &args, int k,
                                 int blocks_per_mod, cudaStream_t stream);
cudaError_t launch_glynn_m32_hi(int N, const M32Args &args, int k,
                                int blocks_per_mod, cudaStream_t stream);
int occupancy_glynn_m32_lo(int N);
int occupancy_glynn_m32_mid(int N);
int occupancy_glynn_m32_hi(int N);
// The same for wide moduli (glynn_m32w_*.cu).
cudaError_t launch_glynn_m32w_lo(int N, const M32Args &args, int k,
                                 int blocks_per_mod, cudaStream_t stream);
cudaError_t launch_glynn_m32w_mid(int N, const M32Args &args, int k,
                                  int blocks_per_mod, cudaStream_t stream);
cudaError_t launch_glynn_m32w_hi(int N, const M32Args &args, int k,
                                 int blocks_per_mod, cudaStream_t stream);
int occupancy_glynn_m32w_lo(int N);
int occupancy_glynn_m32w_mid(int N);
int occupancy_glynn_m32w_hi(int N);

}  // namespace pg
