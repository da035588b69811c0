// Instantiations of the 32-bit Montgomery Glynn kernel for wide moduli
// (2^31 <= p < 2^32) and orders 23..42.
#include "glynn_m32.cuh"

namespace pg {

cudaError_t launch_glynn_m32w_mid(int N, const M32Args &args, int k,
                                 int blocks_per_mod, cudaStream_t stream) {
    switch (N) {
    case 23: return launch_glynn_m32<23, true>(args, k, blocks_per_mod, stream);
    case 24: return launch_glynn_m32<24, true>(args, k, blocks_per_mod, stream);
    case 25: return launch_glynn_m32<25, true>(args, k, blocks_per_mod, stream);
    case 26: return launch_glynn_m32<26, true>(args, k, blocks_per_mod, stream);
    case 27: return launch_glynn_m32<27, true>(args, k, blocks_per_mod, stream);
    case 28: return launch_glynn_m32<28, true>(args, k, blocks_per_mod, stream);
    case 29: return launch_glynn_m32<29, true>(args, k, blocks_per_mod, stream);
    case 30: return launch_glynn_m32<30, true>(args, k, blocks_per_mod, stream);
    case 31: return launch_glynn_m32<31, true>(args, k, blocks_per_mod, stream);
    case 32: return launch_glynn_m32<32, true>(args, k, blocks_per_mod, stream);
    case 33: return launch_glynn_m32<33, true>(args, k, blocks_per_mod, stream);
    case 34: return launch_glynn_m32<34, true>(args, k, blocks_per_mod, stream);
    case 35: return launch_glynn_m32<35, true>(args, k, blocks_per_mod, stream);
    case 36: return launch_glynn_m32<36, true>(args, k, blocks_per_mod, stream);
    case 37: return launch_glynn_m32<37, true>(args, k, blocks_per_mod, stream);
    case 38: return launch_glynn_m32<38, true>(args, k, blocks_per_mod, stream);
    case 39: return launch_glynn_m32<39, true>(args, k, blocks_per_mod, stream);
    case 40: return launch_glynn_m32<40, true>(args, k, blocks_per_mod, stream);
    case 41: return launch_glynn_m32<41, true>(args, k, blocks_per_mod, stream);
    case 42: return launch_glynn_m32<42, true>(args, k, blocks_per_mod, stream);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_glynn_m32w_mid(int N) {
    switch (N) {
    case 23: return occupancy_glynn_m32<23, true>();
    case 24: return occupancy_glynn_m32<24, true>();
    case 25: return occupancy_glynn_m32<25, true>();
    case 26: return occupancy_glynn_m32<26, true>();
    case 27: return occupancy_glynn_m32<27, true>();
    case 28: return occupancy_glynn_m32<28, true>();
    case 29: return occupancy_glynn_m32<29, true>();
    case 30: return occupancy_glynn_m32<30, true>();
    case 31: return occupancy_glynn_m32<31, true>();
    case 32: return occupancy_glynn_m32<32, true>();
    case 33: return occupancy_glynn_m32<33, true>();
    case 34: return occupancy_glynn_m32<34, true>();
    case 35: return occupancy_glynn_m32<35, true>();
    case 36: return occupancy_glynn_m32<36, true>();
    case 37: return occupancy_glynn_m32<37, true>();
    case 38: return occupancy_glynn_m32<38, true>();
    case 39: return occupancy_glynn_m32<39, true>();
    case 40: return occupancy_glynn_m32<40, true>();
    case 41: return occupancy_glynn_m32<41, true>();
    case 42: return occupancy_glynn_m32<42, true>();
    default: return 0;
    }
}

}  // namespace pg
