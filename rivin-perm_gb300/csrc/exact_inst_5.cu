// Instantiations of the exact Glynn kernel (part 5 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_5(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 65:
        if (args) *err = launch_exact_glynn<4, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 1>();
        return true;
    case 113:
        if (args) *err = launch_exact_glynn<7, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 1>();
        return true;
    case 161:
        if (args) *err = launch_exact_glynn<10, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 1>();
        return true;
    case 209:
        if (args) *err = launch_exact_glynn<13, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 1>();
        return true;
    case 257:
        if (args) *err = launch_exact_glynn<16, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 1>();
        return true;
    case 308:
        if (args) *err = launch_exact_glynn<19, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 4>();
        return true;
    case 372:
        if (args) *err = launch_exact_glynn<23, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 4>();
        return true;
    case 405:
        if (args) *err = launch_exact_glynn<25, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 5>();
        return true;
    case 426:
        if (args) *err = launch_exact_glynn<26, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 10>();
        return true;
    case 453:
        if (args) *err = launch_exact_glynn<28, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 5>();
        return true;
    case 474:
        if (args) *err = launch_exact_glynn<29, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 10>();
        return true;
    case 501:
        if (args) *err = launch_exact_glynn<31, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 5>();
        return true;
    case 522:
        if (args) *err = launch_exact_glynn<32, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 10>();
        return true;
    case 551:
        if (args) *err = launch_exact_glynn<34, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 7>();
        return true;
    case 581:
        if (args) *err = launch_exact_glynn<36, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 5>();
        return true;
    case 611:
        if (args) *err = launch_exact_glynn<38, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 3>();
        return true;
    case 632:
        if (args) *err = launch_exact_glynn<39, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 8>();
        return true;
    case 662:
        if (args) *err = launch_exact_glynn<41, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 6>();
        return true;
    case 692:
        if (args) *err = launch_exact_glynn<43, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 4>();
        return true;
    case 714:
        if (args) *err = launch_exact_glynn<44, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 10>();
        return true;
    case 743:
        if (args) *err = launch_exact_glynn<46, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 7>();
        return true;
    case 773:
        if (args) *err = launch_exact_glynn<48, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 5>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
