// Instantiations of the exact Glynn kernel (part 6 of 12),
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_6(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 16 + G) {
    case 66:
        if (args) *err = launch_exact_glynn<4, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 2>();
        return true;
    case 114:
        if (args) *err = launch_exact_glynn<7, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 2>();
        return true;
    case 162:
        if (args) *err = launch_exact_glynn<10, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 2>();
        return true;
    case 210:
        if (args) *err = launch_exact_glynn<13, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 2>();
        return true;
    case 258:
        if (args) *err = launch_exact_glynn<16, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 2>();
        return true;
    case 322:
        if (args) *err = launch_exact_glynn<20, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 2>();
        return true;
    case 386:
        if (args) *err = launch_exact_glynn<24, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 2>();
        return true;
    case 406:
        if (args) *err = launch_exact_glynn<25, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 6>();
        return true;
    case 434:
        if (args) *err = launch_exact_glynn<27, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 2>();
        return true;
    case 454:
        if (args) *err = launch_exact_glynn<28, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 6>();
        return true;
    case 482:
        if (args) *err = launch_exact_glynn<30, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 2>();
        return true;
    case 502:
        if (args) *err = launch_exact_glynn<31, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 6>();
        return true;
    case 531:
        if (args) *err = launch_exact_glynn<33, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 3>();
        return true;
    case 552:
        if (args) *err = launch_exact_glynn<34, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 8>();
        return true;
    case 582:
        if (args) *err = launch_exact_glynn<36, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 6>();
        return true;
    case 612:
        if (args) *err = launch_exact_glynn<38, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 4>();
        return true;
    case 634:
        if (args) *err = launch_exact_glynn<39, 10>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 10>();
        return true;
    case 663:
        if (args) *err = launch_exact_glynn<41, 7>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 7>();
        return true;
    case 693:
        if (args) *err = launch_exact_glynn<43, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 5>();
        return true;
    case 723:
        if (args) *err = launch_exact_glynn<45, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 3>();
        return true;
    case 744:
        if (args) *err = launch_exact_glynn<46, 8>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 8>();
        return true;
    case 774:
        if (args) *err = launch_exact_glynn<48, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 6>();
        return true;
    default:
        return false;
    }
}

}  // namespace pg
