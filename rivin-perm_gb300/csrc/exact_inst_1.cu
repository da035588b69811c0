// Instantiations of the exact Glynn kernel (part 1 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_1(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 34:
        if (args) *err = launch_exact_glynn<2, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<2, 2>();
        return true;
    case 97:
        if (args) *err = launch_exact_glynn<6, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 1>();
        return true;
    case 145:
        if (args) *err = launch_exact_glynn<9, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 1>();
        return true;
    case 193:
        if (args) *err = launch_exact_glynn<12, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 1>();
        return true;
    case 241:
        if (args) *err = launch_exact_glynn<15, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 1>();
        return true;
    case 291:
        if (args) *err = launch_exact_glynn<18, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 3>();
        return true;
    case 355:
        if (args) *err = launch_exact_glynn<22, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 3>();
        return true;
    case 394:
        if (args) *err = launch_exact_glynn<24, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 10>();
        return true;
    case 421:
        if (args) *err = launch_exact_glynn<26, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 5>();
        return true;
    case 442:
        if (args) *err = launch_exact_glynn<27, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 10>();
        return true;
    case 469:
        if (args) *err = launch_exact_glynn<29, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 5>();
        return true;
    case 490:
        if (args) *err = launch_exact_glynn<30, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 10>();
        return true;
    case 517:
        if (args) *err = launch_exact_glynn<32, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 5>();
        return true;
    case 547:
        if (args) *err = launch_exact_glynn<34, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 3>();
        return true;
    case 568:
        if (args) *err = launch_exact_glynn<35, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 8>();
        return true;
    case 598:
        if (args) *err = launch_exact_glynn<37, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 6>();
        return true;
    case 628:
        if (args) *err = launch_exact_glynn<39, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 4>();
        return true;
    case 650:
        if (args) *err = launch_exact_glynn<40, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 10>();
        return true;
    case 679:
        if (args) *err = launch_exact_glynn<42, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 7>();
        return true;
    case 709:
        if (args) *err = launch_exact_glynn<44, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 5>();
        return true;
    case 739:
        if (args) *err = launch_exact_glynn<46, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 3>();
        return true;
    case 760:
        if (args) *err = launch_exact_glynn<47, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 8>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
