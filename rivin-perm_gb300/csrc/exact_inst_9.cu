// Instantiations of the exact Glynn kernel (part 9 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_9(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 81:
        if (args) *err = launch_exact_glynn<5, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 1>();
        return true;
    case 129:
        if (args) *err = launch_exact_glynn<8, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 1>();
        return true;
    case 177:
        if (args) *err = launch_exact_glynn<11, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 1>();
        return true;
    case 225:
        if (args) *err = launch_exact_glynn<14, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 1>();
        return true;
    case 274:
        if (args) *err = launch_exact_glynn<17, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 2>();
        return true;
    case 338:
        if (args) *err = launch_exact_glynn<21, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 2>();
        return true;
    case 389:
        if (args) *err = launch_exact_glynn<24, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 5>();
        return true;
    case 410:
        if (args) *err = launch_exact_glynn<25, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 10>();
        return true;
    case 437:
        if (args) *err = launch_exact_glynn<27, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 5>();
        return true;
    case 458:
        if (args) *err = launch_exact_glynn<28, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 10>();
        return true;
    case 485:
        if (args) *err = launch_exact_glynn<30, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 5>();
        return true;
    case 506:
        if (args) *err = launch_exact_glynn<31, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 10>();
        return true;
    case 534:
        if (args) *err = launch_exact_glynn<33, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 6>();
        return true;
    case 564:
        if (args) *err = launch_exact_glynn<35, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 4>();
        return true;
    case 586:
        if (args) *err = launch_exact_glynn<36, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 10>();
        return true;
    case 615:
        if (args) *err = launch_exact_glynn<38, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 7>();
        return true;
    case 645:
        if (args) *err = launch_exact_glynn<40, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 5>();
        return true;
    case 675:
        if (args) *err = launch_exact_glynn<42, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 3>();
        return true;
    case 696:
        if (args) *err = launch_exact_glynn<43, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 8>();
        return true;
    case 726:
        if (args) *err = launch_exact_glynn<45, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 6>();
        return true;
    case 756:
        if (args) *err = launch_exact_glynn<47, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 4>();
        return true;
    case 778:
        if (args) *err = launch_exact_glynn<48, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 10>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
