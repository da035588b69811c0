// Runtime plumbing for the permgpu C ABI: per-thread error text, device
// query, per-thread stream + scratch workspace, the host-mapped abort word and
// the Gray-chunk planner.
#include "pg_internal.h"

#include <mutex>
#include <string>

namespace pg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int status, const std::string &msg) {
    set_error(msg);
    return status;
}

int cuda_fail(cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                    cudaGetErrorString(e) + ")";
    set_error(m);
    if (e == cudaErrorMemoryAllocation) return PG_ENOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return PG_ENODEV;
    return PG_ECUDA;
}

int device_info(DeviceInfo *out) {
    static std::mutex mu;
    static DeviceInfo cached;
    static bool have = false;
    std::lock_guard<std::mutex> lock(mu);
    if (!have) {
        int count = 0;
        cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0)
            return fail(PG_ENODEV, "no CUDA device visible");
        DeviceInfo d;
        PG_CUDA(cudaGetDevice(&d.device));
        PG_CUDA(cudaDeviceGetAttribute(&d.sm_count,
                                       cudaDevAttrMultiProcessorCount, d.device));
        PG_CUDA(cudaDeviceGetAttribute(&d.cc_major,
                                       cudaDevAttrComputeCapabilityMajor, d.device));
        PG_CUDA(cudaDeviceGetAttribute(&d.cc_minor,
                                       cudaDevAttrComputeCapabilityMinor, d.device));
        int optin = 0;
        PG_CUDA(cudaDeviceGetAttribute(&optin,
                                       cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                       d.device));
        d.smem_optin = (size_t)optin;
        cached = d;
        have = true;
    }
    *out = cached;
    return PG_OK;
}

struct WorkspaceHolder {
    Workspace ws;
    ~WorkspaceHolder() {
        // Runs at thread exit; the CUDA context may already be gone at
        // process exit, so errors are ignored here.
        if (ws.dev) cudaFree(ws.dev);
        if (ws.host) cudaFreeHost(ws.host);
        if (ws.stream) cudaStreamDestroy(ws.stream);
    }
};
static thread_local WorkspaceHolder g_ws;

int workspace(Workspace **out, size_t dev_bytes, size_t host_bytes) {
    Workspace &ws = g_ws.ws;
    if (!ws.stream) {
        PG_CUDA(cudaStreamCreateWithFlags(&ws.stream, cudaStreamNonBlocking));
    }
    if (dev_bytes > ws.dev_bytes) {
        if (ws.dev) {
            PG_CUDA(cudaStreamSynchronize(ws.stream));
            PG_CUDA(cudaFree(ws.dev));
            ws.dev = nullptr;
            ws.dev_bytes = 0;
        }
        size_t want = dev_bytes < 4096 ? 4096 : dev_bytes;
        PG_CUDA(cudaMalloc(&ws.dev, want));
        ws.dev_bytes = want;
    }
    if (host_bytes > ws.host_bytes) {
        if (ws.host) {
            PG_CUDA(cudaStreamSynchronize(ws.stream));
            PG_CUDA(cudaFreeHost(ws.host));
            ws.host = nullptr;
            ws.host_bytes = 0;
        }
        size_t want = host_bytes < 4096 ? 4096 : host_bytes;
        PG_CUDA(cudaHostAlloc(&ws.host, want, cudaHostAllocDefault));
        ws.host_bytes = want;
    }
    *out = &ws;
    return PG_OK;
}

static volatile int *g_abort_host = nullptr;
static volatile int *g_abort_dev = nullptr;
static std::mutex g_abort_mu;

int abort_flag_device(volatile int **dptr) {
    std::lock_guard<std::mutex> lock(g_abort_mu);
    if (!g_abort_host) {
        void *h = nullptr;
        PG_CUDA(cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped));
        *(volatile int *)h = 0;
        void *d = nullptr;
        PG_CUDA(cudaHostGetDevicePointer(&d, h, 0));
        g_abort_host = (volatile int *)h;
        g_abort_dev = (volatile int *)d;
    }
    *dptr = g_abort_dev;
    return PG_OK;
}

volatile int *abort_flag_device_if_created() {
    std::lock_guard<std::mutex> lock(g_abort_mu);
    return g_abort_dev;
}

ChunkPlan plan_chunks(int log_states, int min_log_len, uint64_t target_chunks) {
    // Largest chunk count that is a power of two <= target, keeping chunks at
    // least 2^min_log_len long and at most 2^30 (accumulator headroom), and
    // at most 2^24 chunks (reduction headroom).
    ChunkPlan pl;
    int log_chunks = 0;
    while ((2ull << log_chunks) <= target_chunks) log_chunks++;
    int log_len = log_states - log_chunks;
    if (log_len < min_log_len) log_len = min_log_len;
    if (log_len > log_states) log_len = log_states;
    if (log_states - log_len > 24) log_len = log_states - 24;
    if (log_len > 30) log_len = 30;
    pl.log_len = log_len;
    pl.chunks = 1ull << (log_states - log_len);
    return pl;
}

}  // namespace pg

extern "C" {

int pg_version(void) { return 100; }

const char *pg_last_error(void) { return pg::g_last_error.c_str(); }

int pg_cuda_runtime_available(void) {
    pg::DeviceInfo d;
    return pg::device_info(&d) == PG_OK ? 1 : 0;
}

int pg_device_info(int *sm_count, int *cc_major, int *cc_minor) {
    pg::DeviceInfo d;
    int st = pg::device_info(&d);
    if (st != PG_OK) return st;
    if (sm_count) *sm_count = d.sm_count;
    if (cc_major) *cc_major = d.cc_major;
    if (cc_minor) *cc_minor = d.cc_minor;
    return PG_OK;
}

void pg_abort(void) {
    volatile int *d;
    if (pg::abort_flag_device(&d) == PG_OK && pg::g_abort_host)
        *pg::g_abort_host = 1;
}

void pg_clear_abort(void) {
    volatile int *d;
    if (pg::abort_flag_device(&d) == PG_OK && pg::g_abort_host)
        *pg::g_abort_host = 0;
}

}  // extern "C"
