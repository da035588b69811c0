// Instantiations of the exact Glynn kernel (part 11 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_11(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 83:
        if (args) *err = launch_exact_glynn<5, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 3>();
        return true;
    case 131:
        if (args) *err = launch_exact_glynn<8, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 3>();
        return true;
    case 179:
        if (args) *err = launch_exact_glynn<11, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 3>();
        return true;
    case 227:
        if (args) *err = launch_exact_glynn<14, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 3>();
        return true;
    case 276:
        if (args) *err = launch_exact_glynn<17, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 4>();
        return true;
    case 340:
        if (args) *err = launch_exact_glynn<21, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 4>();
        return true;
    case 391:
        if (args) *err = launch_exact_glynn<24, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 7>();
        return true;
    case 419:
        if (args) *err = launch_exact_glynn<26, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 3>();
        return true;
    case 439:
        if (args) *err = launch_exact_glynn<27, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 7>();
        return true;
    case 467:
        if (args) *err = launch_exact_glynn<29, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 3>();
        return true;
    case 487:
        if (args) *err = launch_exact_glynn<30, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 7>();
        return true;
    case 515:
        if (args) *err = launch_exact_glynn<32, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 3>();
        return true;
    case 536:
        if (args) *err = launch_exact_glynn<33, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 8>();
        return true;
    case 566:
        if (args) *err = launch_exact_glynn<35, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 6>();
        return true;
    case 596:
        if (args) *err = launch_exact_glynn<37, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 4>();
        return true;
    case 618:
        if (args) *err = launch_exact_glynn<38, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 10>();
        return true;
    case 647:
        if (args) *err = launch_exact_glynn<40, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 7>();
        return true;
    case 677:
        if (args) *err = launch_exact_glynn<42, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 5>();
        return true;
    case 707:
        if (args) *err = launch_exact_glynn<44, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 3>();
        return true;
    case 728:
        if (args) *err = launch_exact_glynn<45, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 8>();
        return true;
    case 758:
        if (args) *err = launch_exact_glynn<47, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 6>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
