// Instantiations of the exact Glynn kernel (part 0 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_0(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 33:
        if (args) *err = launch_exact_glynn<2, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<2, 1>();
        return true;
    case 84:
        if (args) *err = launch_exact_glynn<5, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 4>();
        return true;
    case 132:
        if (args) *err = launch_exact_glynn<8, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 4>();
        return true;
    case 180:
        if (args) *err = launch_exact_glynn<11, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 4>();
        return true;
    case 228:
        if (args) *err = launch_exact_glynn<14, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 4>();
        return true;
    case 290:
        if (args) *err = launch_exact_glynn<18, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 2>();
        return true;
    case 354:
        if (args) *err = launch_exact_glynn<22, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 2>();
        return true;
    case 392:
        if (args) *err = launch_exact_glynn<24, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 8>();
        return true;
    case 420:
        if (args) *err = launch_exact_glynn<26, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 4>();
        return true;
    case 440:
        if (args) *err = launch_exact_glynn<27, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 8>();
        return true;
    case 468:
        if (args) *err = launch_exact_glynn<29, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 4>();
        return true;
    case 488:
        if (args) *err = launch_exact_glynn<30, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 8>();
        return true;
    case 516:
        if (args) *err = launch_exact_glynn<32, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 4>();
        return true;
    case 538:
        if (args) *err = launch_exact_glynn<33, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 10>();
        return true;
    case 567:
        if (args) *err = launch_exact_glynn<35, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 7>();
        return true;
    case 597:
        if (args) *err = launch_exact_glynn<37, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 5>();
        return true;
    case 627:
        if (args) *err = launch_exact_glynn<39, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 3>();
        return true;
    case 648:
        if (args) *err = launch_exact_glynn<40, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 8>();
        return true;
    case 678:
        if (args) *err = launch_exact_glynn<42, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 6>();
        return true;
    case 708:
        if (args) *err = launch_exact_glynn<44, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 4>();
        return true;
    case 730:
        if (args) *err = launch_exact_glynn<45, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 10>();
        return true;
    case 759:
        if (args) *err = launch_exact_glynn<47, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 7>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
