// Instantiations of the exact Glynn kernel (part 2 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_2(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 49:
        if (args) *err = launch_exact_glynn<3, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 1>();
        return true;
    case 98:
        if (args) *err = launch_exact_glynn<6, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 2>();
        return true;
    case 146:
        if (args) *err = launch_exact_glynn<9, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 2>();
        return true;
    case 194:
        if (args) *err = launch_exact_glynn<12, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 2>();
        return true;
    case 242:
        if (args) *err = launch_exact_glynn<15, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 2>();
        return true;
    case 292:
        if (args) *err = launch_exact_glynn<18, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 4>();
        return true;
    case 356:
        if (args) *err = launch_exact_glynn<22, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 4>();
        return true;
    case 402:
        if (args) *err = launch_exact_glynn<25, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 2>();
        return true;
    case 422:
        if (args) *err = launch_exact_glynn<26, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 6>();
        return true;
    case 450:
        if (args) *err = launch_exact_glynn<28, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 2>();
        return true;
    case 470:
        if (args) *err = launch_exact_glynn<29, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 6>();
        return true;
    case 498:
        if (args) *err = launch_exact_glynn<31, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 2>();
        return true;
    case 518:
        if (args) *err = launch_exact_glynn<32, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 6>();
        return true;
    case 548:
        if (args) *err = launch_exact_glynn<34, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 4>();
        return true;
    case 570:
        if (args) *err = launch_exact_glynn<35, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 10>();
        return true;
    case 599:
        if (args) *err = launch_exact_glynn<37, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 7>();
        return true;
    case 629:
        if (args) *err = launch_exact_glynn<39, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 5>();
        return true;
    case 659:
        if (args) *err = launch_exact_glynn<41, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 3>();
        return true;
    case 680:
        if (args) *err = launch_exact_glynn<42, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 8>();
        return true;
    case 710:
        if (args) *err = launch_exact_glynn<44, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 6>();
        return true;
    case 740:
        if (args) *err = launch_exact_glynn<46, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 4>();
        return true;
    case 762:
        if (args) *err = launch_exact_glynn<47, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 10>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
