// Instantiations of the 32-bit Montgomery Glynn kernel for orders 23..42.
#include "glynn_m32.cuh"

namespace pg {

cudaError_t launch_glynn_m32_mid(int N, const M32Args &args, int k,
                                  int blocks_per_mod, cudaStream_t stream) {
    switch (N) {
    case 23: return launch_glynn_m32<23>(args, k, blocks_per_mod, stream);
    case 24: return launch_glynn_m32<24>(args, k, blocks_per_mod, stream);
    case 25: return launch_glynn_m32<25>(args, k, blocks_per_mod, stream);
    case 26: return launch_glynn_m32<26>(args, k, blocks_per_mod, stream);
    case 27: return launch_glynn_m32<27>(args, k, blocks_per_mod, stream);
    case 28: return launch_glynn_m32<28>(args, k, blocks_per_mod, stream);
    case 29: return launch_glynn_m32<29>(args, k, blocks_per_mod, stream);
    case 30: return launch_glynn_m32<30>(args, k, blocks_per_mod, stream);
    case 31: return launch_glynn_m32<31>(args, k, blocks_per_mod, stream);
    case 32: return launch_glynn_m32<32>(args, k, blocks_per_mod, stream);
    case 33: return launch_glynn_m32<33>(args, k, blocks_per_mod, stream);
    case 34: return launch_glynn_m32<34>(args, k, blocks_per_mod, stream);
    case 35: return launch_glynn_m32<35>(args, k, blocks_per_mod, stream);
    case 36: return launch_glynn_m32<36>(args, k, blocks_per_mod, stream);
    case 37: return launch_glynn_m32<37>(args, k, blocks_per_mod, stream);
    case 38: return launch_glynn_m32<38>(args, k, blocks_per_mod, stream);
    case 39: return launch_glynn_m32<39>(args, k, blocks_per_mod, stream);
    case 40: return launch_glynn_m32<40>(args, k, blocks_per_mod, stream);
    case 41: return launch_glynn_m32<41>(args, k, blocks_per_mod, stream);
    case 42: return launch_glynn_m32<42>(args, k, blocks_per_mod, stream);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_glynn_m32_mid(int N) {
    switch (N) {
    case 23: return occupancy_glynn_m32<23>();
    case 24: return occupancy_glynn_m32<24>();
    case 25: return occupancy_glynn_m32<25>();
    case 26: return occupancy_glynn_m32<26>();
    case 27: return occupancy_glynn_m32<27>();
    case 28: return occupancy_glynn_m32<28>();
    case 29: return occupancy_glynn_m32<29>();
    case 30: return occupancy_glynn_m32<30>();
    case 31: return occupancy_glynn_m32<31>();
    case 32: return occupancy_glynn_m32<32>();
    case 33: return occupancy_glynn_m32<33>();
    case 34: return occupancy_glynn_m32<34>();
    case 35: return occupancy_glynn_m32<35>();
    case 36: return occupancy_glynn_m32<36>();
    case 37: return occupancy_glynn_m32<37>();
    case 38: return occupancy_glynn_m32<38>();
    case 39: return occupancy_glynn_m32<39>();
    case 40: return occupancy_glynn_m32<40>();
    case 41: return occupancy_glynn_m32<41>();
    case 42: return occupancy_glynn_m32<42>();
    default: return 0;
    }
}

}  // namespace pg
