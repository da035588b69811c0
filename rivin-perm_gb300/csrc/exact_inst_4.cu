// Instantiations of the exact Glynn kernel (part 4 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_4(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 51:
        if (args) *err = launch_exact_glynn<3, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 3>();
        return true;
    case 100:
        if (args) *err = launch_exact_glynn<6, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 4>();
        return true;
    case 148:
        if (args) *err = launch_exact_glynn<9, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 4>();
        return true;
    case 196:
        if (args) *err = launch_exact_glynn<12, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 4>();
        return true;
    case 244:
        if (args) *err = launch_exact_glynn<15, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 4>();
        return true;
    case 307:
        if (args) *err = launch_exact_glynn<19, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 3>();
        return true;
    case 371:
        if (args) *err = launch_exact_glynn<23, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 3>();
        return true;
    case 404:
        if (args) *err = launch_exact_glynn<25, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 4>();
        return true;
    case 424:
        if (args) *err = launch_exact_glynn<26, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 8>();
        return true;
    case 452:
        if (args) *err = launch_exact_glynn<28, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 4>();
        return true;
    case 472:
        if (args) *err = launch_exact_glynn<29, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 8>();
        return true;
    case 500:
        if (args) *err = launch_exact_glynn<31, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 4>();
        return true;
    case 520:
        if (args) *err = launch_exact_glynn<32, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 8>();
        return true;
    case 550:
        if (args) *err = launch_exact_glynn<34, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 6>();
        return true;
    case 580:
        if (args) *err = launch_exact_glynn<36, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 4>();
        return true;
    case 602:
        if (args) *err = launch_exact_glynn<37, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 10>();
        return true;
    case 631:
        if (args) *err = launch_exact_glynn<39, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 7>();
        return true;
    case 661:
        if (args) *err = launch_exact_glynn<41, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 5>();
        return true;
    case 691:
        if (args) *err = launch_exact_glynn<43, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 3>();
        return true;
    case 712:
        if (args) *err = launch_exact_glynn<44, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 8>();
        return true;
    case 742:
        if (args) *err = launch_exact_glynn<46, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 6>();
        return true;
    case 772:
        if (args) *err = launch_exact_glynn<48, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 4>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
