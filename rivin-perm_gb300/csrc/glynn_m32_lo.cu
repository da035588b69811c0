// Instantiations of the 32-bit Montgomery Glynn kernel for orders 2..22.
#include "glynn_m32.cuh"

namespace pg {

cudaError_t launch_glynn_m32_lo(int N, const M32Args &args, int k,
                                  int blocks_per_mod, cudaStream_t stream) {
    switch (N) {
    case 2: return launch_glynn_m32<2>(args, k, blocks_per_mod, stream);
    case 3: return launch_glynn_m32<3>(args, k, blocks_per_mod, stream);
    case 4: return launch_glynn_m32<4>(args, k, blocks_per_mod, stream);
    case 5: return launch_glynn_m32<5>(args, k, blocks_per_mod, stream);
    case 6: return launch_glynn_m32<6>(args, k, blocks_per_mod, stream);
    case 7: return launch_glynn_m32<7>(args, k, blocks_per_mod, stream);
    case 8: return launch_glynn_m32<8>(args, k, blocks_per_mod, stream);
    case 9: return launch_glynn_m32<9>(args, k, blocks_per_mod, stream);
    case 10: return launch_glynn_m32<10>(args, k, blocks_per_mod, stream);
    case 11: return launch_glynn_m32<11>(args, k, blocks_per_mod, stream);
    case 12: return launch_glynn_m32<12>(args, k, blocks_per_mod, stream);
    case 13: return launch_glynn_m32<13>(args, k, blocks_per_mod, stream);
    case 14: return launch_glynn_m32<14>(args, k, blocks_per_mod, stream);
    case 15: return launch_glynn_m32<15>(args, k, blocks_per_mod, stream);
    case 16: return launch_glynn_m32<16>(args, k, blocks_per_mod, stream);
    case 17: return launch_glynn_m32<17>(args, k, blocks_per_mod, stream);
    case 18: return launch_glynn_m32<18>(args, k, blocks_per_mod, stream);
    case 19: return launch_glynn_m32<19>(args, k, blocks_per_mod, stream);
    case 20: return launch_glynn_m32<20>(args, k, blocks_per_mod, stream);
    case 21: return launch_glynn_m32<21>(args, k, blocks_per_mod, stream);
    case 22: return launch_glynn_m32<22>(args, k, blocks_per_mod, stream);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_glynn_m32_lo(int N) {
    switch (N) {
    case 2: return occupancy_glynn_m32<2>();
    case 3: return occupancy_glynn_m32<3>();
    case 4: return occupancy_glynn_m32<4>();
    case 5: return occupancy_glynn_m32<5>();
    case 6: return occupancy_glynn_m32<6>();
    case 7: return occupancy_glynn_m32<7>();
    case 8: return occupancy_glynn_m32<8>();
    case 9: return occupancy_glynn_m32<9>();
    case 10: return occupancy_glynn_m32<10>();
    case 11: return occupancy_glynn_m32<11>();
    case 12: return occupancy_glynn_m32<12>();
    case 13: return occupancy_glynn_m32<13>();
    case 14: return occupancy_glynn_m32<14>();
    case 15: return occupancy_glynn_m32<15>();
    case 16: return occupancy_glynn_m32<16>();
    case 17: return occupancy_glynn_m32<17>();
    case 18: return occupancy_glynn_m32<18>();
    case 19: return occupancy_glynn_m32<19>();
    case 20: return occupancy_glynn_m32<20>();
    case 21: return occupancy_glynn_m32<21>();
    case 22: return occupancy_glynn_m32<22>();
    default: return 0;
    }
}

}  // namespace pg
