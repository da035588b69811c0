// Instantiations of the 32-bit Montgomery Glynn kernel for wide moduli
// (2^31 <= p < 2^32) and orders 43..63.
#include "glynn_m32.cuh"

namespace pg {

cudaError_t launch_glynn_m32w_hi(int N, const M32Args &args, int k,
                                 int blocks_per_mod, cudaStream_t stream) {
    switch (N) {
    case 43: return launch_glynn_m32<43, true>(args, k, blocks_per_mod, stream);
    case 44: return launch_glynn_m32<44, true>(args, k, blocks_per_mod, stream);
    case 45: return launch_glynn_m32<45, true>(args, k, blocks_per_mod, stream);
    case 46: return launch_glynn_m32<46, true>(args, k, blocks_per_mod, stream);
    case 47: return launch_glynn_m32<47, true>(args, k, blocks_per_mod, stream);
    case 48: return launch_glynn_m32<48, true>(args, k, blocks_per_mod, stream);
    case 49: return launch_glynn_m32<49, true>(args, k, blocks_per_mod, stream);
    case 50: return launch_glynn_m32<50, true>(args, k, blocks_per_mod, stream);
    case 51: return launch_glynn_m32<51, true>(args, k, blocks_per_mod, stream);
    case 52: return launch_glynn_m32<52, true>(args, k, blocks_per_mod, stream);
    case 53: return launch_glynn_m32<53, true>(args, k, blocks_per_mod, stream);
    case 54: return launch_glynn_m32<54, true>(args, k, blocks_per_mod, stream);
    case 55: return launch_glynn_m32<55, true>(args, k, blocks_per_mod, stream);
    case 56: return launch_glynn_m32<56, true>(args, k, blocks_per_mod, stream);
    case 57: return launch_glynn_m32<57, true>(args, k, blocks_per_mod, stream);
    case 58: return launch_glynn_m32<58, true>(args, k, blocks_per_mod, stream);
    case 59: return launch_glynn_m32<59, true>(args, k, blocks_per_mod, stream);
    case 60: return launch_glynn_m32<60, true>(args, k, blocks_per_mod, stream);
    case 61: return launch_glynn_m32<61, true>(args, k, blocks_per_mod, stream);
    case 62: return launch_glynn_m32<62, true>(args, k, blocks_per_mod, stream);
    case 63: return launch_glynn_m32<63, true>(args, k, blocks_per_mod, stream);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_glynn_m32w_hi(int N) {
    switch (N) {
    case 43: return occupancy_glynn_m32<43, true>();
    case 44: return occupancy_glynn_m32<44, true>();
    case 45: return occupancy_glynn_m32<45, true>();
    case 46: return occupancy_glynn_m32<46, true>();
    case 47: return occupancy_glynn_m32<47, true>();
    case 48: return occupancy_glynn_m32<48, true>();
    case 49: return occupancy_glynn_m32<49, true>();
    case 50: return occupancy_glynn_m32<50, true>();
    case 51: return occupancy_glynn_m32<51, true>();
    case 52: return occupancy_glynn_m32<52, true>();
    case 53: return occupancy_glynn_m32<53, true>();
    case 54: return occupancy_glynn_m32<54, true>();
    case 55: return occupancy_glynn_m32<55, true>();
    case 56: return occupancy_glynn_m32<56, true>();
    case 57: return occupancy_glynn_m32<57, true>();
    case 58: return occupancy_glynn_m32<58, true>();
    case 59: return occupancy_glynn_m32<59, true>();
    case 60: return occupancy_glynn_m32<60, true>();
    case 61: return occupancy_glynn_m32<61, true>();
    case 62: return occupancy_glynn_m32<62, true>();
    case 63: return occupancy_glynn_m32<63, true>();
    default: return 0;
    }
}

}  // namespace pg
