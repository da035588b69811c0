// Instantiations of the exact Glynn kernel (part 3 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_3(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 50:
        if (args) *err = launch_exact_glynn<3, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 2>();
        return true;
    case 99:
        if (args) *err = launch_exact_glynn<6, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 3>();
        return true;
    case 147:
        if (args) *err = launch_exact_glynn<9, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 3>();
        return true;
    case 195:
        if (args) *err = launch_exact_glynn<12, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 3>();
        return true;
    case 243:
        if (args) *err = launch_exact_glynn<15, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 3>();
        return true;
    case 306:
        if (args) *err = launch_exact_glynn<19, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 2>();
        return true;
    case 370:
        if (args) *err = launch_exact_glynn<23, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 2>();
        return true;
    case 403:
        if (args) *err = launch_exact_glynn<25, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 3>();
        return true;
    case 423:
        if (args) *err = launch_exact_glynn<26, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 7>();
        return true;
    case 451:
        if (args) *err = launch_exact_glynn<28, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 3>();
        return true;
    case 471:
        if (args) *err = launch_exact_glynn<29, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 7>();
        return true;
    case 499:
        if (args) *err = launch_exact_glynn<31, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 3>();
        return true;
    case 519:
        if (args) *err = launch_exact_glynn<32, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 7>();
        return true;
    case 549:
        if (args) *err = launch_exact_glynn<34, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 5>();
        return true;
    case 579:
        if (args) *err = launch_exact_glynn<36, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 3>();
        return true;
    case 600:
        if (args) *err = launch_exact_glynn<37, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 8>();
        return true;
    case 630:
        if (args) *err = launch_exact_glynn<39, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 6>();
        return true;
    case 660:
        if (args) *err = launch_exact_glynn<41, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 4>();
        return true;
    case 682:
        if (args) *err = launch_exact_glynn<42, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 10>();
        return true;
    case 711:
        if (args) *err = launch_exact_glynn<44, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 7>();
        return true;
    case 741:
        if (args) *err = launch_exact_glynn<46, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 5>();
        return true;
    case 771:
        if (args) *err = launch_exact_glynn<48, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 3>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
