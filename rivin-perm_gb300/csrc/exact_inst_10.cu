// Instantiations of the exact Glynn kernel (part 10 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_10(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 82:
        if (args) *err = launch_exact_glynn<5, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 2>();
        return true;
    case 130:
        if (args) *err = launch_exact_glynn<8, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 2>();
        return true;
    case 178:
        if (args) *err = launch_exact_glynn<11, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 2>();
        return true;
    case 226:
        if (args) *err = launch_exact_glynn<14, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 2>();
        return true;
    case 275:
        if (args) *err = launch_exact_glynn<17, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 3>();
        return true;
    case 339:
        if (args) *err = launch_exact_glynn<21, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 3>();
        return true;
    case 390:
        if (args) *err = launch_exact_glynn<24, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 6>();
        return true;
    case 418:
        if (args) *err = launch_exact_glynn<26, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 2>();
        return true;
    case 438:
        if (args) *err = launch_exact_glynn<27, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 6>();
        return true;
    case 466:
        if (args) *err = launch_exact_glynn<29, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 2>();
        return true;
    case 486:
        if (args) *err = launch_exact_glynn<30, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 6>();
        return true;
    case 514:
        if (args) *err = launch_exact_glynn<32, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 2>();
        return true;
    case 535:
        if (args) *err = launch_exact_glynn<33, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 7>();
        return true;
    case 565:
        if (args) *err = launch_exact_glynn<35, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 5>();
        return true;
    case 595:
        if (args) *err = launch_exact_glynn<37, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 3>();
        return true;
    case 616:
        if (args) *err = launch_exact_glynn<38, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 8>();
        return true;
    case 646:
        if (args) *err = launch_exact_glynn<40, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 6>();
        return true;
    case 676:
        if (args) *err = launch_exact_glynn<42, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 4>();
        return true;
    case 698:
        if (args) *err = launch_exact_glynn<43, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 10>();
        return true;
    case 727:
        if (args) *err = launch_exact_glynn<45, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 7>();
        return true;
    case 757:
        if (args) *err = launch_exact_glynn<47, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 5>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
