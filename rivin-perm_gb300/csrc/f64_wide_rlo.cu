// Instantiations of glynn_wide_kernel: real matrices, orders 2..32.
#include "f64_wide.cuh"

namespace pg {

cudaError_t launch_glynn_wide_real_lo(int n, const WideArgs &a, cudaStream_t s) {
    switch (n) {
    case 2: return launch_glynn_wide<2, false>(a, s);
    case 3: return launch_glynn_wide<3, false>(a, s);
    case 4: return launch_glynn_wide<4, false>(a, s);
    case 5: return launch_glynn_wide<5, false>(a, s);
    case 6: return launch_glynn_wide<6, false>(a, s);
    case 7: return launch_glynn_wide<7, false>(a, s);
    case 8: return launch_glynn_wide<8, false>(a, s);
    case 9: return launch_glynn_wide<9, false>(a, s);
    case 10: return launch_glynn_wide<10, false>(a, s);
    case 11: return launch_glynn_wide<11, false>(a, s);
    case 12: return launch_glynn_wide<12, false>(a, s);
    case 13: return launch_glynn_wide<13, false>(a, s);
    case 14: return launch_glynn_wide<14, false>(a, s);
    case 15: return launch_glynn_wide<15, false>(a, s);
    case 16: return launch_glynn_wide<16, false>(a, s);
    case 17: return launch_glynn_wide<17, false>(a, s);
    case 18: return launch_glynn_wide<18, false>(a, s);
    case 19: return launch_glynn_wide<19, false>(a, s);
    case 20: return launch_glynn_wide<20, false>(a, s);
    case 21: return launch_glynn_wide<21, false>(a, s);
    case 22: return launch_glynn_wide<22, false>(a, s);
    case 23: return launch_glynn_wide<23, false>(a, s);
    case 24: return launch_glynn_wide<24, false>(a, s);
    case 25: return launch_glynn_wide<25, false>(a, s);
    case 26: return launch_glynn_wide<26, false>(a, s);
    case 27: return launch_glynn_wide<27, false>(a, s);
    case 28: return launch_glynn_wide<28, false>(a, s);
    case 29: return launch_glynn_wide<29, false>(a, s);
    case 30: return launch_glynn_wide<30, false>(a, s);
    case 31: return launch_glynn_wide<31, false>(a, s);
    case 32: return launch_glynn_wide<32, false>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace pg
