// Pipe throughput probe: the denominators of the integer and FP32 rooflines.
//
// Each thread runs 8 independent dependency chains of one PTX multiply-add
// form for `iters` iterations over a grid of 4 x SMs blocks x 256 threads,
// timed with CUDA events.  Variants:
//   0  mad.lo.u32   (32-bit multiply-add, low word)
//   1  mad.wide.u32 (32x32 -> 64-bit multiply-add; one ALU prmt beside it)
//   2  mad.hi.u32   (high word)
//   3  add.u32      (integer ALU add, for the mix reference)
//   4  mul.wide.u32 (32x32 -> 64-bit product, no addend; one ALU xor beside it)
//   5  fma.rn.f32   (FP32 fused multiply-add: the double-float kernels' pipe)
//   6  fma.rn.f64   (FP64 fused multiply-add)
// Returns operations per second (one op = one instruction for one thread).
// A measurement utility: the bench divides by these rates; no engine calls it.
#include "pg_internal.h"

namespace pg {

template <int V>
__global__ void __launch_bounds__(256) imad_probe_kernel(uint32_t seed, int iters,
                                                         uint32_t *sink) {
    uint32_t x[8], y = seed * 2654435761u + threadIdx.x;
    uint64_t w[8];
    float f[8];
    double dd[8];
    const float fy = 0.999f + 1e-7f * (float)(threadIdx.x & 7);
    const double dy = 0.999 + 1e-9 * (double)(threadIdx.x & 7);
#pragma unroll
    for (int c = 0; c < 8; c++) {
        x[c] = seed + c * 977u + threadIdx.x;
        w[c] = x[c];
        f[c] = 1.0f + 0.01f * (float)c;
        dd[c] = 1.0 + 0.01 * (double)c;
    }
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < 8; c++) {
            if (V == 0) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(x[c]) : "r"(y), "r"(c + 1u));
            // the multiplicand is byte-rotated every iteration (prmt, an
            // ALU-pipe instruction independent of the running sum), so no
            // product can be hoisted, the only dependency through the sum is
            // the 64-bit addend, and the IMAD pipe executes only the mad.wide
            if (V == 1)
                asm volatile("prmt.b32 %1, %1, 0, 0x0321;\n\t"
                             "mad.wide.u32 %0, %1, %2, %0;"
                             : "+l"(w[c]), "+r"(x[c]) : "r"(y));
            if (V == 2) asm volatile("mad.hi.u32 %0, %0, %1, %2;" : "+r"(x[c]) : "r"(y), "r"(c + 7u));
            // mul.wide.u32 without an addend: the next multiplicand is the
            // XOR of the product's halves (one ALU-pipe lop3)
            if (V == 4)
                asm volatile("{\n\t.reg .u64 t;\n\t.reg .u32 lo, hi;\n\t"
                             "mul.wide.u32 t, %0, %1;\n\t"
                             "mov.b64 {lo, hi}, t;\n\t"
                             "xor.b32 %0, lo, hi;\n\t}"
                             : "+r"(x[c]) : "r"(y));
            if (V == 3) asm volatile("add.u32 %0, %0, %1;" : "+r"(x[c]) : "r"(y));
            if (V == 5) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(f[c]) : "f"(fy), "f"(1e-3f));
            if (V == 6) asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(dd[c]) : "d"(dy), "d"(1e-3));
        }
    }
    uint32_t acc = 0;
#pragma unroll
    for (int c = 0; c < 8; c++)
        acc ^= x[c] ^ (uint32_t)w[c] ^ (uint32_t)(w[c] >> 32) ^ __float_as_uint(f[c]) ^
               (uint32_t)__double_as_longlong(dd[c]);
    if (acc == 0x9e3779b9u) sink[0] = acc;   // keeps the chains live
}

}  // namespace pg

extern "C" int pg_probe_int_throughput(int variant, int iters, double *ops_per_second) {
    using namespace pg;
    if (!ops_per_second || variant < 0 || variant > 6 || iters < 1)
        return fail(PG_EINVAL, "bad probe arguments");
    DeviceInfo dev;
    int st = device_info(&dev);
    if (st != PG_OK) return st;
    Workspace *ws;
    st = workspace(&ws, 64, 64);
    if (st != PG_OK) return st;
    const int blocks = dev.sm_count * 4;
    cudaEvent_t a, b;
    PG_CUDA(cudaEventCreate(&a));
    PG_CUDA(cudaEventCreate(&b));
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        PG_CUDA(cudaEventRecord(a, ws->stream));
        uint32_t *sink = (uint32_t *)ws->dev;
        switch (variant) {
        case 0: imad_probe_kernel<0><<<blocks, 256, 0, ws->stream>>>(rep, iters, sink); break;
        case 1: imad_probe_kernel<1><<<blocks, 256, 0, ws->stream>>>(rep, iters, sink); break;
        case 2: imad_probe_kernel<2><<<blocks, 256, 0, ws->stream>>>(rep, iters, sink); break;
        case 4: imad_probe_kernel<4><<<blocks, 256, 0, ws->stream>>>(rep, iters, sink); break;
        case 5: imad_probe_kernel<5><<<blocks, 256, 0, ws->stream>>>(rep, iters, sink); break;
        case 6: imad_probe_kernel<6><<<blocks, 256, 0, ws->stream>>>(rep, iters, sink); break;
        default: imad_probe_kernel<3><<<blocks, 256, 0, ws->stream>>>(rep, iters, sink); break;
        }
        PG_CUDA(cudaGetLastError());
        PG_CUDA(cudaEventRecord(b, ws->stream));
        PG_CUDA(cudaEventSynchronize(b));
        float ms = 0;
        PG_CUDA(cudaEventElapsedTime(&ms, a, b));
        if (rep > 0 && ms < best) best = ms;   // first launch is warm-up
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const double ops = (double)blocks * 256.0 * 8.0 * (double)iters;
    *ops_per_second = ops / (best * 1e-3);
    return PG_OK;
}
