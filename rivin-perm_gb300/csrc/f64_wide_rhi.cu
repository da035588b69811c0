// Instantiations of glynn_wide_kernel: real matrices, orders 33..63.
#include "f64_wide.cuh"

namespace pg {

cudaError_t launch_glynn_wide_real_hi(int n, const WideArgs &a, cudaStream_t s) {
    switch (n) {
    case 33: return launch_glynn_wide<33, false>(a, s);
    case 34: return launch_glynn_wide<34, false>(a, s);
    case 35: return launch_glynn_wide<35, false>(a, s);
    case 36: return launch_glynn_wide<36, false>(a, s);
    case 37: return launch_glynn_wide<37, false>(a, s);
    case 38: return launch_glynn_wide<38, false>(a, s);
    case 39: return launch_glynn_wide<39, false>(a, s);
    case 40: return launch_glynn_wide<40, false>(a, s);
    case 41: return launch_glynn_wide<41, false>(a, s);
    case 42: return launch_glynn_wide<42, false>(a, s);
    case 43: return launch_glynn_wide<43, false>(a, s);
    case 44: return launch_glynn_wide<44, false>(a, s);
    case 45: return launch_glynn_wide<45, false>(a, s);
    case 46: return launch_glynn_wide<46, false>(a, s);
    case 47: return launch_glynn_wide<47, false>(a, s);
    case 48: return launch_glynn_wide<48, false>(a, s);
    case 49: return launch_glynn_wide<49, false>(a, s);
    case 50: return launch_glynn_wide<50, false>(a, s);
    case 51: return launch_glynn_wide<51, false>(a, s);
    case 52: return launch_glynn_wide<52, false>(a, s);
    case 53: return launch_glynn_wide<53, false>(a, s);
    case 54: return launch_glynn_wide<54, false>(a, s);
    case 55: return launch_glynn_wide<55, false>(a, s);
    case 56: return launch_glynn_wide<56, false>(a, s);
    case 57: return launch_glynn_wide<57, false>(a, s);
    case 58: return launch_glynn_wide<58, false>(a, s);
    case 59: return launch_glynn_wide<59, false>(a, s);
    case 60: return launch_glynn_wide<60, false>(a, s);
    case 61: return launch_glynn_wide<61, false>(a, s);
    case 62: return launch_glynn_wide<62, false>(a, s);
    case 63: return launch_glynn_wide<63, false>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace pg
