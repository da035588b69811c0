// Instantiations of the exact Glynn kernel (part 7 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_7(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 67:
        if (args) *err = launch_exact_glynn<4, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 3>();
        return true;
    case 115:
        if (args) *err = launch_exact_glynn<7, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 3>();
        return true;
    case 163:
        if (args) *err = launch_exact_glynn<10, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 3>();
        return true;
    case 211:
        if (args) *err = launch_exact_glynn<13, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 3>();
        return true;
    case 259:
        if (args) *err = launch_exact_glynn<16, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 3>();
        return true;
    case 323:
        if (args) *err = launch_exact_glynn<20, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 3>();
        return true;
    case 387:
        if (args) *err = launch_exact_glynn<24, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 3>();
        return true;
    case 407:
        if (args) *err = launch_exact_glynn<25, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 7>();
        return true;
    case 435:
        if (args) *err = launch_exact_glynn<27, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 3>();
        return true;
    case 455:
        if (args) *err = launch_exact_glynn<28, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 7>();
        return true;
    case 483:
        if (args) *err = launch_exact_glynn<30, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 3>();
        return true;
    case 503:
        if (args) *err = launch_exact_glynn<31, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 7>();
        return true;
    case 532:
        if (args) *err = launch_exact_glynn<33, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 4>();
        return true;
    case 554:
        if (args) *err = launch_exact_glynn<34, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 10>();
        return true;
    case 583:
        if (args) *err = launch_exact_glynn<36, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 7>();
        return true;
    case 613:
        if (args) *err = launch_exact_glynn<38, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 5>();
        return true;
    case 643:
        if (args) *err = launch_exact_glynn<40, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 3>();
        return true;
    case 664:
        if (args) *err = launch_exact_glynn<41, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 8>();
        return true;
    case 694:
        if (args) *err = launch_exact_glynn<43, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 6>();
        return true;
    case 724:
        if (args) *err = launch_exact_glynn<45, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 4>();
        return true;
    case 746:
        if (args) *err = launch_exact_glynn<46, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 10>();
        return true;
    case 775:
        if (args) *err = launch_exact_glynn<48, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 7>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
