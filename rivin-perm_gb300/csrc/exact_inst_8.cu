// Instantiations of the exact Glynn kernel (part 8 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_8(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 68:
        if (args) *err = launch_exact_glynn<4, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 4>();
        return true;
    case 116:
        if (args) *err = launch_exact_glynn<7, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 4>();
        return true;
    case 164:
        if (args) *err = launch_exact_glynn<10, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 4>();
        return true;
    case 212:
        if (args) *err = launch_exact_glynn<13, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 4>();
        return true;
    case 260:
        if (args) *err = launch_exact_glynn<16, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 4>();
        return true;
    case 324:
        if (args) *err = launch_exact_glynn<20, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 4>();
        return true;
    case 388:
        if (args) *err = launch_exact_glynn<24, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 4>();
        return true;
    case 408:
        if (args) *err = launch_exact_glynn<25, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 8>();
        return true;
    case 436:
        if (args) *err = launch_exact_glynn<27, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 4>();
        return true;
    case 456:
        if (args) *err = launch_exact_glynn<28, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 8>();
        return true;
    case 484:
        if (args) *err = launch_exact_glynn<30, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 4>();
        return true;
    case 504:
        if (args) *err = launch_exact_glynn<31, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 8>();
        return true;
    case 533:
        if (args) *err = launch_exact_glynn<33, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 5>();
        return true;
    case 563:
        if (args) *err = launch_exact_glynn<35, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 3>();
        return true;
    case 584:
        if (args) *err = launch_exact_glynn<36, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 8>();
        return true;
    case 614:
        if (args) *err = launch_exact_glynn<38, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 6>();
        return true;
    case 644:
        if (args) *err = launch_exact_glynn<40, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 4>();
        return true;
    case 666:
        if (args) *err = launch_exact_glynn<41, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 10>();
        return true;
    case 695:
        if (args) *err = launch_exact_glynn<43, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 7>();
        return true;
    case 725:
        if (args) *err = launch_exact_glynn<45, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 5>();
        return true;
    case 755:
        if (args) *err = launch_exact_glynn<47, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 3>();
        return true;
    case 776:
        if (args) *err = launch_exact_glynn<48, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 8>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
