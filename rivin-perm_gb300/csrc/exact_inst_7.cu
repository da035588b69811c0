// Instantiations of the exact Glynn kernel (part 7 of 8).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_7(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 35:
        if (args) *err = launch_exact_glynn<4, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 3>();
        return true;
    case 51:
        if (args) *err = launch_exact_glynn<6, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 3>();
        return true;
    case 67:
        if (args) *err = launch_exact_glynn<8, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 3>();
        return true;
    case 83:
        if (args) *err = launch_exact_glynn<10, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 3>();
        return true;
    case 99:
        if (args) *err = launch_exact_glynn<12, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 3>();
        return true;
    case 115:
        if (args) *err = launch_exact_glynn<14, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 3>();
        return true;
    case 131:
        if (args) *err = launch_exact_glynn<16, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 3>();
        return true;
    case 154:
        if (args) *err = launch_exact_glynn<19, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 2>();
        return true;
    case 172:
        if (args) *err = launch_exact_glynn<21, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 4>();
        return true;
    case 195:
        if (args) *err = launch_exact_glynn<24, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 3>();
        return true;
    case 206:
        if (args) *err = launch_exact_glynn<25, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 6>();
        return true;
    case 220:
        if (args) *err = launch_exact_glynn<27, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 4>();
        return true;
    case 234:
        if (args) *err = launch_exact_glynn<29, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 2>();
        return true;
    case 245:
        if (args) *err = launch_exact_glynn<30, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 5>();
        return true;
    case 259:
        if (args) *err = launch_exact_glynn<32, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 3>();
        return true;
    case 275:
        if (args) *err = launch_exact_glynn<34, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 3>();
        return true;
    case 291:
        if (args) *err = launch_exact_glynn<36, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 3>();
        return true;
    case 307:
        if (args) *err = launch_exact_glynn<38, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 3>();
        return true;
    case 323:
        if (args) *err = launch_exact_glynn<40, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 3>();
        return true;
    case 339:
        if (args) *err = launch_exact_glynn<42, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 3>();
        return true;
    case 355:
        if (args) *err = launch_exact_glynn<44, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 3>();
        return true;
    case 371:
        if (args) *err = launch_exact_glynn<46, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 3>();
        return true;
    case 387:
        if (args) *err = launch_exact_glynn<48, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 3>();
        return true;
    default: return false;
    }
}

}  // namespace pg
