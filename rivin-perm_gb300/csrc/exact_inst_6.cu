// Instantiations of the exact Glynn kernel (part 6 of 8).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_6(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 34:
        if (args) *err = launch_exact_glynn<4, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 2>();
        return true;
    case 50:
        if (args) *err = launch_exact_glynn<6, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 2>();
        return true;
    case 66:
        if (args) *err = launch_exact_glynn<8, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 2>();
        return true;
    case 82:
        if (args) *err = launch_exact_glynn<10, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 2>();
        return true;
    case 98:
        if (args) *err = launch_exact_glynn<12, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 2>();
        return true;
    case 114:
        if (args) *err = launch_exact_glynn<14, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 2>();
        return true;
    case 130:
        if (args) *err = launch_exact_glynn<16, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 2>();
        return true;
    case 148:
        if (args) *err = launch_exact_glynn<18, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 4>();
        return true;
    case 171:
        if (args) *err = launch_exact_glynn<21, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 3>();
        return true;
    case 194:
        if (args) *err = launch_exact_glynn<24, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 2>();
        return true;
    case 205:
        if (args) *err = launch_exact_glynn<25, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 5>();
        return true;
    case 219:
        if (args) *err = launch_exact_glynn<27, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 3>();
        return true;
    case 230:
        if (args) *err = launch_exact_glynn<28, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 6>();
        return true;
    case 244:
        if (args) *err = launch_exact_glynn<30, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 4>();
        return true;
    case 258:
        if (args) *err = launch_exact_glynn<32, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 2>();
        return true;
    case 270:
        if (args) *err = launch_exact_glynn<33, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 6>();
        return true;
    case 286:
        if (args) *err = launch_exact_glynn<35, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 6>();
        return true;
    case 302:
        if (args) *err = launch_exact_glynn<37, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 6>();
        return true;
    case 318:
        if (args) *err = launch_exact_glynn<39, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 6>();
        return true;
    case 334:
        if (args) *err = launch_exact_glynn<41, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 6>();
        return true;
    case 350:
        if (args) *err = launch_exact_glynn<43, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 6>();
        return true;
    case 366:
        if (args) *err = launch_exact_glynn<45, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 6>();
        return true;
    case 382:
        if (args) *err = launch_exact_glynn<47, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 6>();
        return true;
    default: return false;
    }
}

}  // namespace pg
