// Instantiations of the 32-bit Montgomery Glynn kernel for orders 43..63.
#include "glynn_m32.cuh"

namespace pg {

cudaError_t launch_glynn_m32_hi(int N, const M32Args &args, int k,
                                  int blocks_per_mod, cudaStream_t stream) {
    switch (N) {
    case 43: return launch_glynn_m32<43>(args, k, blocks_per_mod, stream);
    case 44: return launch_glynn_m32<44>(args, k, blocks_per_mod, stream);
    case 45: return launch_glynn_m32<45>(args, k, blocks_per_mod, stream);
    case 46: return launch_glynn_m32<46>(args, k, blocks_per_mod, stream);
    case 47: return launch_glynn_m32<47>(args, k, blocks_per_mod, stream);
    case 48: return launch_glynn_m32<48>(args, k, blocks_per_mod, stream);
    case 49: return launch_glynn_m32<49>(args, k, blocks_per_mod, stream);
    case 50: return launch_glynn_m32<50>(args, k, blocks_per_mod, stream);
    case 51: return launch_glynn_m32<51>(args, k, blocks_per_mod, stream);
    case 52: return launch_glynn_m32<52>(args, k, blocks_per_mod, stream);
    case 53: return launch_glynn_m32<53>(args, k, blocks_per_mod, stream);
    case 54: return launch_glynn_m32<54>(args, k, blocks_per_mod, stream);
    case 55: return launch_glynn_m32<55>(args, k, blocks_per_mod, stream);
    case 56: return launch_glynn_m32<56>(args, k, blocks_per_mod, stream);
    case 57: return launch_glynn_m32<57>(args, k, blocks_per_mod, stream);
    case 58: return launch_glynn_m32<58>(args, k, blocks_per_mod, stream);
    case 59: return launch_glynn_m32<59>(args, k, blocks_per_mod, stream);
    case 60: return launch_glynn_m32<60>(args, k, blocks_per_mod, stream);
    case 61: return launch_glynn_m32<61>(args, k, blocks_per_mod, stream);
    case 62: return launch_glynn_m32<62>(args, k, blocks_per_mod, stream);
    case 63: return launch_glynn_m32<63>(args, k, blocks_per_mod, stream);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_glynn_m32_hi(int N) {
    switch (N) {
    case 43: return occupancy_glynn_m32<43>();
    case 44: return occupancy_glynn_m32<44>();
    case 45: return occupancy_glynn_m32<45>();
    case 46: return occupancy_glynn_m32<46>();
    case 47: return occupancy_glynn_m32<47>();
    case 48: return occupancy_glynn_m32<48>();
    case 49: return occupancy_glynn_m32<49>();
    case 50: return occupancy_glynn_m32<50>();
    case 51: return occupancy_glynn_m32<51>();
    case 52: return occupancy_glynn_m32<52>();
    case 53: return occupancy_glynn_m32<53>();
    case 54: return occupancy_glynn_m32<54>();
    case 55: return occupancy_glynn_m32<55>();
    case 56: return occupancy_glynn_m32<56>();
    case 57: return occupancy_glynn_m32<57>();
    case 58: return occupancy_glynn_m32<58>();
    case 59: return occupancy_glynn_m32<59>();
    case 60: return occupancy_glynn_m32<60>();
    case 61: return occupancy_glynn_m32<61>();
    case 62: return occupancy_glynn_m32<62>();
    case 63: return occupancy_glynn_m32<63>();
    default: return 0;
    }
}

}  // namespace pg
