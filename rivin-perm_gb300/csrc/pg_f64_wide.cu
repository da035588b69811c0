// Host side of the FP64 window kernel (f64_wide.cuh): launch shape, slot
// reduction and the C entry point pg_glynn_window.  pg_f64.cu sends whole
// walks of orders 33..63 here.
#include "pg_internal.h"
#include "f64_wide.cuh"

#include <cmath>
#include <vector>

namespace pg {

// One block per matrix; lane l Kahan-sums the slots l, l + 32, ... and
// lane 0 adds the 32 partial sums in lane order (deterministic).  Undoes
// the row scaling and the term shift; whole walks also divide by 2^(n-1).
__global__ void glynn_wide_reduce(const double *Are, const double *Aim, const double *slots,
                                  int n, int log_w, int shift, int whole, double *re,
                                  double *im, double *abs_sum) {
    const int b = blockIdx.x, lane = threadIdx.x;
    const int W = 1 << log_w;
    const double *base = slots + (size_t)b * W * WIDE_SLOT;
    double sr = 0, cr = 0, si = 0, ci = 0, as = 0;
    for (int w = lane; w < W; w += 32) {
        const double *sl = base + (size_t)w * WIDE_SLOT;
        kahan(sr, cr, sl[0]);
        kahan(sr, cr, -sl[1]);
        kahan(si, ci, sl[2]);
        kahan(si, ci, -sl[3]);
        as += sl[4];
    }
    __shared__ double part[32][3];
    part[lane][0] = sr - cr;
    part[lane][1] = si - ci;
    part[lane][2] = as;
    __syncwarp();
    if (lane != 0) return;
    int et = 0;
    for (int i = 0; i < n; i++) {
        double rowsum = 0.0;
        for (int j = 0; j < n; j++) {
            rowsum += fabs(Are[(size_t)b * n * n + i * n + j]);
            if (Aim) rowsum += fabs(Aim[(size_t)b * n * n + i * n + j]);
        }
        int e = 0;
        if (rowsum > 0.0) { frexp(rowsum, &e); e = -e; }
        et += e;
    }
    double tr = 0, tcr = 0, ti = 0, tci = 0, ta = 0;
    for (int l = 0; l < 32; l++) {
        kahan(tr, tcr, part[l][0]);
        kahan(ti, tci, part[l][1]);
        ta += part[l][2];
    }
    const int sc = -et - shift - (whole ? n - 1 : 0);
    re[b] = ldexp(tr, sc);
    if (im) im[b] = ldexp(ti, sc);
    if (abs_sum) abs_sum[b] = ldexp(ta, sc);
}

static cudaError_t launch_wide_any(int n, bool cplx, const WideArgs &a, cudaStream_t s) {
    if (n >= 2 && n <= 32) return cplx ? launch_glynn_wide_cplx_lo(n, a, s)
                                       : launch_glynn_wide_real_lo(n, a, s);
    if (n >= 33 && n <= 63) return cplx ? launch_glynn_wide_cplx_hi(n, a, s)
                                        : launch_glynn_wide_real_hi(n, a, s);
    return cudaErrorInvalidValue;
}

int glynn_wide_run(const double *Are, const double *Aim, int batch, int n, uint64_t lo,
                   uint64_t count, bool whole, double *re, double *im, double *abs_sum,
                   cudaStream_t stream) {
    if (n < 2 || n > 63) return fail(PG_ERANGE, "FP64 window kernel supports 2 <= n <= 63");
    if (batch <= 0 || count == 0) return PG_OK;
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    volatile int *abort_dev;
    st = abort_flag_device(&abort_dev);
    if (st != PG_OK) return st;
    // warps per matrix: about 80 per SM overall while every warp keeps at
    // least 2^12 states (one exact re-initialisation period)
    int log_w = 0;
    while (log_w < 24 && (((long)batch << log_w) < (long)dev.sm_count * 80) &&
           (count >> (log_w + 1)) >= (1ull << 12))
        log_w++;
    int log_block = 0;
    while (log_block < 12 && (2ull << log_block) <= (count >> log_w)) log_block++;
    const size_t slots = (size_t)batch << log_w;
    const size_t bytes = slots * WIDE_SLOT * sizeof(double) + 256;
    Workspace *ws;
    st = workspace(&ws, bytes, 64);
    if (st != PG_OK) return st;
    cudaStream_t s = stream ? stream : ws->stream;
    int *status = (int *)((char *)ws->dev + bytes - 256);
    PG_CUDA(cudaMemsetAsync(ws->dev, 0, bytes, s));
    WideArgs a;
    a.Are = Are;
    a.Aim = Aim;
    a.batch = batch;
    a.log_w = log_w;
    a.wpb = log_w >= 2 ? 4 : 1 << log_w;
    a.log_block = log_block;
    a.g_lo = lo;
    a.g_count = count;
    a.slots = (double *)ws->dev;
    a.abort_flag = abort_dev;
    a.status = status;
    PG_CUDA(launch_wide_any(n, Aim != nullptr, a, s));
    glynn_wide_reduce<<<batch, 32, 0, s>>>(Are, Aim, (const double *)ws->dev, n, log_w,
                                           wide_shift(n), whole ? 1 : 0, re, im, abs_sum);
    PG_CUDA(cudaGetLastError());
    int hstatus = 0;
    PG_CUDA(cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    if (hstatus) return fail(PG_EABORT, "FP64 window launch aborted by pg_abort()");
    return PG_OK;
}

}  // namespace pg

extern "C" int pg_glynn_window(const double *Are, const double *Aim, int n, uint64_t lo,
                               uint64_t hi, double *sum_re, double *sum_im, double *abs_sum) {
    using namespace pg;
    if (n < 2 || n > 63) return fail(PG_ERANGE, "FP64 window kernel supports 2 <= n <= 63");
    if (!Are || !sum_re) return fail(PG_EINVAL, "null argument");
    const uint64_t states = 1ull << (n - 1);
    if (lo > hi || hi > states) return fail(PG_ERANGE, "window must satisfy lo <= hi <= 2^(n-1)");
    if (lo == hi) {
        *sum_re = 0.0;
        if (sum_im) *sum_im = 0.0;
        if (abs_sum) *abs_sum = 0.0;
        return PG_OK;
    }
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    const size_t na = (size_t)n * n;
    const bool cplx = Aim != nullptr;
    double *d = nullptr;
    PG_CUDA(cudaMalloc(&d, (na * (cplx ? 2 : 1) + 3) * sizeof(double)));
    double *dre = d, *dim = cplx ? d + na : nullptr;
    double *dout = d + na * (cplx ? 2 : 1);
    cudaError_t e = cudaMemcpy(dre, Are, na * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && cplx) e = cudaMemcpy(dim, Aim, na * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "cudaMemcpy(A)");
    }
    st = glynn_wide_run(dre, dim, 1, n, lo, hi - lo, false, dout, dout + 1, dout + 2, nullptr);
    double h[3] = {0, 0, 0};
    if (st == PG_OK) {
        e = cudaMemcpy(h, dout, sizeof(h), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpy(results)");
    }
    cudaFree(d);
    if (st != PG_OK) return st;
    *sum_re = h[0];
    if (sum_im) *sum_im = h[1];
    if (abs_sum) *abs_sum = h[2];
    return PG_OK;
}
