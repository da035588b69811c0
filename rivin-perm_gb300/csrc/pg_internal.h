// Internal helpers shared by the permgpu translation units: status/error
// plumbing, per-thread device workspace, the abort flag and the Gray-code
// chunk plan used by every traversal kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <string>

#include "../../include/permgpu.h"

namespace pg {

// ---- error plumbing -------------------------------------------------------
void set_error(const std::string &msg);
int fail(int status, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define PG_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t _e = (call);                                             \
        if (_e != cudaSuccess) return ::pg::cuda_fail(_e, #call);            \
    } while (0)

// ---- device / workspace ---------------------------------------------------
struct DeviceInfo {
    int device = -1;
    int sm_count = 0;
    int cc_major = 0, cc_minor = 0;
    size_t smem_optin = 0;
};
// Initialises the CUDA context on first use.  Returns PG_OK or an error.
int device_info(DeviceInfo *out);

// Per-host-thread stream and grow-only device/pinned-host scratch.  The
// buffers are reused across calls from the same thread.
struct Workspace {
    cudaStream_t stream = nullptr;
    void *dev = nullptr;
    size_t dev_bytes = 0;
    void *host = nullptr;
    size_t host_bytes = 0;
};
int workspace(Workspace **ws, size_t dev_bytes, size_t host_bytes);

// Device pointer of the host-mapped abort word (0 = run, 1 = abort).
int abort_flag_device(volatile int **dptr);
// The same pointer when an earlier call already created the word, else
// nullptr; never allocates.
volatile int *abort_flag_device_if_created();

// ---- chunk plan -----------------------------------------------------------
// A traversal of 2^s Gray states is cut into 2^(s-log_len) aligned chunks of
// 2^log_len states.  Alignment makes the toggled column at local step i
// equal ctz(i) for every chunk, so all lanes of a warp read the same column.
struct ChunkPlan {
    int log_len;        // chunk length 2^log_len
    uint64_t chunks;    // chunks per traversal
};
ChunkPlan plan_chunks(int log_states, int min_log_len, uint64_t target_chunks);

// ---- host modular helpers (exact, 128-bit) -------------------------------
static inline uint64_t mulmod_u64(uint64_t a, uint64_t b, uint64_t m) {
    return (uint64_t)(((unsigned __int128)a * b) % m);
}
static inline uint64_t powmod_u64(uint64_t b, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    b %= m;
    while (e) {
        if (e & 1) r = mulmod_u64(r, b, m);
        b = mulmod_u64(b, b, m);
        e >>= 1;
    }
    return r;
}
static inline uint64_t normmod_i64(int64_t v, uint64_t m) {
    // exact for the full int64 range
    __int128 r = (__int128)v % (__int128)m;
    if (r < 0) r += m;
    return (uint64_t)r;
}
// -m^{-1} mod 2^32 / 2^64 for odd m (Newton iteration)
static inline uint32_t neg_inv32(uint32_t m) {
    uint32_t x = m;  // correct to 3 bits
    for (int i = 0; i < 5; i++) x *= 2u - m * x;
    return (uint32_t)(0u - x);
}
static inline uint64_t neg_inv64(uint64_t m) {
    uint64_t x = m;
    for (int i = 0; i < 6; i++) x *= 2u - m * x;
    return (uint64_t)(0u - x);
}

// ---- residue engine entry points (pg_residue*.cu) ------------------------
// Mod-p Glynn over an arbitrary residue matrix for a batch of odd moduli.
// `mats` holds k row-major n x n matrices with entries already in [0, m_t).
// out[t] = per(mats[t]) mod m_t.
int glynn_residues_odd(const uint64_t *mats, int n, const uint64_t *moduli,
                       int k, uint64_t *out);
// Ryser in Z/2^64 (wrap-around) for the power-of-two part of even moduli.
int ryser_wrap64(const int64_t *A, int n, uint64_t *out);

// ---- necklace quotient for Schur permanents of prime order (pg_necklace.cu)
// Moduli must be odd and below this bound (lazy row sums, see pg_necklace.cu).
constexpr uint64_t NECKLACE_PRIME_LIMIT = 1ull << 30;
// Smallest order the automatic Schur dispatch sends to the necklace kernel;
// below it the Glynn cofactor kernel finishes first.
constexpr int NECKLACE_AUTO_MIN_ORDER = 37;
// Odd moduli 2^30 <= p < 2^32 take the wide-modulus necklace kernel, which
// is compiled for the orders of necklace_wide_supported (n >= 37).
constexpr uint64_t NECKLACE_WIDE_PRIME_LIMIT = 1ull << 32;
// True when n - 1 is a compiled necklace minor order (n an odd prime < 64).
bool necklace_supported(int n);
// True when the wide-modulus necklace kernel is compiled for order n.
bool necklace_wide_supported(int n);
// out[t] = perm(S_n) mod primes[t] for odd primes[t] < NECKLACE_PRIME_LIMIT
// (< NECKLACE_WIDE_PRIME_LIMIT when necklace_wide_supported(n)) with
// omegas[t]^n == 1; n must satisfy necklace_supported(n).
int schur_necklace_residues(int n, const uint64_t *primes, const uint64_t *omegas, int k,
                            uint64_t *out);

}  // namespace pg
