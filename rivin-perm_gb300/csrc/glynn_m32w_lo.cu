// Instantiations of the 32-bit Montgomery Glynn kernel for wide moduli
// (2^31 <= p < 2^32) and orders 2..22.
#include "glynn_m32.cuh"

namespace pg {

cudaError_t launch_glynn_m32w_lo(int N, const M32Args &args, int k,
                                 int blocks_per_mod, cudaStream_t stream) {
    switch (N) {
    case 2: return launch_glynn_m32<2, true>(args, k, blocks_per_mod, stream);
    case 3: return launch_glynn_m32<3, true>(args, k, blocks_per_mod, stream);
    case 4: return launch_glynn_m32<4, true>(args, k, blocks_per_mod, stream);
    case 5: return launch_glynn_m32<5, true>(args, k, blocks_per_mod, stream);
    case 6: return launch_glynn_m32<6, true>(args, k, blocks_per_mod, stream);
    case 7: return launch_glynn_m32<7, true>(args, k, blocks_per_mod, stream);
    case 8: return launch_glynn_m32<8, true>(args, k, blocks_per_mod, stream);
    case 9: return launch_glynn_m32<9, true>(args, k, blocks_per_mod, stream);
    case 10: return launch_glynn_m32<10, true>(args, k, blocks_per_mod, stream);
    case 11: return launch_glynn_m32<11, true>(args, k, blocks_per_mod, stream);
    case 12: return launch_glynn_m32<12, true>(args, k, blocks_per_mod, stream);
    case 13: return launch_glynn_m32<13, true>(args, k, blocks_per_mod, stream);
    case 14: return launch_glynn_m32<14, true>(args, k, blocks_per_mod, stream);
    case 15: return launch_glynn_m32<15, true>(args, k, blocks_per_mod, stream);
    case 16: return launch_glynn_m32<16, true>(args, k, blocks_per_mod, stream);
    case 17: return launch_glynn_m32<17, true>(args, k, blocks_per_mod, stream);
    case 18: return launch_glynn_m32<18, true>(args, k, blocks_per_mod, stream);
    case 19: return launch_glynn_m32<19, true>(args, k, blocks_per_mod, stream);
    case 20: return launch_glynn_m32<20, true>(args, k, blocks_per_mod, stream);
    case 21: return launch_glynn_m32<21, true>(args, k, blocks_per_mod, stream);
    case 22: return launch_glynn_m32<22, true>(args, k, blocks_per_mod, stream);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_glynn_m32w_lo(int N) {
    switch (N) {
    case 2: return occupancy_glynn_m32<2, true>();
    case 3: return occupancy_glynn_m32<3, true>();
    case 4: return occupancy_glynn_m32<4, true>();
    case 5: return occupancy_glynn_m32<5, true>();
    case 6: return occupancy_glynn_m32<6, true>();
    case 7: return occupancy_glynn_m32<7, true>();
    case 8: return occupancy_glynn_m32<8, true>();
    case 9: return occupancy_glynn_m32<9, true>();
    case 10: return occupancy_glynn_m32<10, true>();
    case 11: return occupancy_glynn_m32<11, true>();
    case 12: return occupancy_glynn_m32<12, true>();
    case 13: return occupancy_glynn_m32<13, true>();
    case 14: return occupancy_glynn_m32<14, true>();
    case 15: return occupancy_glynn_m32<15, true>();
    case 16: return occupancy_glynn_m32<16, true>();
    case 17: return occupancy_glynn_m32<17, true>();
    case 18: return occupancy_glynn_m32<18, true>();
    case 19: return occupancy_glynn_m32<19, true>();
    case 20: return occupancy_glynn_m32<20, true>();
    case 21: return occupancy_glynn_m32<21, true>();
    case 22: return occupancy_glynn_m32<22, true>();
    default: return 0;
    }
}

}  // namespace pg
