// Instantiations of glynn_wide_kernel: complex matrices, orders 2..32.
#include "f64_wide.cuh"

namespace pg {

cudaError_t launch_glynn_wide_cplx_lo(int n, const WideArgs &a, cudaStream_t s) {
    switch (n) {
    case 2: return launch_glynn_wide<2, true>(a, s);
    case 3: return launch_glynn_wide<3, true>(a, s);
    case 4: return launch_glynn_wide<4, true>(a, s);
    case 5: return launch_glynn_wide<5, true>(a, s);
    case 6: return launch_glynn_wide<6, true>(a, s);
    case 7: return launch_glynn_wide<7, true>(a, s);
    case 8: return launch_glynn_wide<8, true>(a, s);
    case 9: return launch_glynn_wide<9, true>(a, s);
    case 10: return launch_glynn_wide<10, true>(a, s);
    case 11: return launch_glynn_wide<11, true>(a, s);
    case 12: return launch_glynn_wide<12, true>(a, s);
    case 13: return launch_glynn_wide<13, true>(a, s);
    case 14: return launch_glynn_wide<14, true>(a, s);
    case 15: return launch_glynn_wide<15, true>(a, s);
    case 16: return launch_glynn_wide<16, true>(a, s);
    case 17: return launch_glynn_wide<17, true>(a, s);
    case 18: return launch_glynn_wide<18, true>(a, s);
    case 19: return launch_glynn_wide<19, true>(a, s);
    case 20: return launch_glynn_wide<20, true>(a, s);
    case 21: return launch_glynn_wide<21, true>(a, s);
    case 22: return launch_glynn_wide<22, true>(a, s);
    case 23: return launch_glynn_wide<23, true>(a, s);
    case 24: return launch_glynn_wide<24, true>(a, s);
    case 25: return launch_glynn_wide<25, true>(a, s);
    case 26: return launch_glynn_wide<26, true>(a, s);
    case 27: return launch_glynn_wide<27, true>(a, s);
    case 28: return launch_glynn_wide<28, true>(a, s);
    case 29: return launch_glynn_wide<29, true>(a, s);
    case 30: return launch_glynn_wide<30, true>(a, s);
    case 31: return launch_glynn_wide<31, true>(a, s);
    case 32: return launch_glynn_wide<32, true>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace pg
