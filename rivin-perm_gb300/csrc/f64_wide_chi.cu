// Instantiations of glynn_wide_kernel: complex matrices, orders 33..63.
#include "f64_wide.cuh"

namespace pg {

cudaError_t launch_glynn_wide_cplx_hi(int n, const WideArgs &a, cudaStream_t s) {
    switch (n) {
    case 33: return launch_glynn_wide<33, true>(a, s);
    case 34: return launch_glynn_wide<34, true>(a, s);
    case 35: return launch_glynn_wide<35, true>(a, s);
    case 36: return launch_glynn_wide<36, true>(a, s);
    case 37: return launch_glynn_wide<37, true>(a, s);
    case 38: return launch_glynn_wide<38, true>(a, s);
    case 39: return launch_glynn_wide<39, true>(a, s);
    case 40: return launch_glynn_wide<40, true>(a, s);
    case 41: return launch_glynn_wide<41, true>(a, s);
    case 42: return launch_glynn_wide<42, true>(a, s);
    case 43: return launch_glynn_wide<43, true>(a, s);
    case 44: return launch_glynn_wide<44, true>(a, s);
    case 45: return launch_glynn_wide<45, true>(a, s);
    case 46: return launch_glynn_wide<46, true>(a, s);
    case 47: return launch_glynn_wide<47, true>(a, s);
    case 48: return launch_glynn_wide<48, true>(a, s);
    case 49: return launch_glynn_wide<49, true>(a, s);
    case 50: return launch_glynn_wide<50, true>(a, s);
    case 51: return launch_glynn_wide<51, true>(a, s);
    case 52: return launch_glynn_wide<52, true>(a, s);
    case 53: return launch_glynn_wide<53, true>(a, s);
    case 54: return launch_glynn_wide<54, true>(a, s);
    case 55: return launch_glynn_wide<55, true>(a, s);
    case 56: return launch_glynn_wide<56, true>(a, s);
    case 57: return launch_glynn_wide<57, true>(a, s);
    case 58: return launch_glynn_wide<58, true>(a, s);
    case 59: return launch_glynn_wide<59, true>(a, s);
    case 60: return launch_glynn_wide<60, true>(a, s);
    case 61: return launch_glynn_wide<61, true>(a, s);
    case 62: return launch_glynn_wide<62, true>(a, s);
    case 63: return launch_glynn_wide<63, true>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace pg
