// Instantiations of the exact Glynn kernel (part 3 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_3(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 52:
        if (args) *err = launch_exact_glynn<3, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 2, false>();
        return true;
    case 87:
        if (args) *err = launch_exact_glynn<5, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 3, true>();
        return true;
    case 119:
        if (args) *err = launch_exact_glynn<7, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 3, true>();
        return true;
    case 151:
        if (args) *err = launch_exact_glynn<9, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 3, true>();
        return true;
    case 183:
        if (args) *err = launch_exact_glynn<11, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 3, true>();
        return true;
    case 215:
        if (args) *err = launch_exact_glynn<13, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 3, true>();
        return true;
    case 247:
        if (args) *err = launch_exact_glynn<15, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 3, true>();
        return true;
    case 281:
        if (args) *err = launch_exact_glynn<17, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 4, true>();
        return true;
    case 326:
        if (args) *err = launch_exact_glynn<20, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 3, false>();
        return true;
    case 359:
        if (args) *err = launch_exact_glynn<22, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 3, true>();
        return true;
    case 391:
        if (args) *err = launch_exact_glynn<24, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 3, true>();
        return true;
    case 413:
        if (args) *err = launch_exact_glynn<25, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 6, true>();
        return true;
    case 440:
        if (args) *err = launch_exact_glynn<27, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 4, false>();
        return true;
    case 455:
        if (args) *err = launch_exact_glynn<28, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 3, true>();
        return true;
    case 477:
        if (args) *err = launch_exact_glynn<29, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 6, true>();
        return true;
    case 504:
        if (args) *err = launch_exact_glynn<31, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 4, false>();
        return true;
    case 519:
        if (args) *err = launch_exact_glynn<32, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 3, true>();
        return true;
    case 550:
        if (args) *err = launch_exact_glynn<34, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 3, false>();
        return true;
    case 567:
        if (args) *err = launch_exact_glynn<35, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 3, true>();
        return true;
    case 598:
        if (args) *err = launch_exact_glynn<37, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 3, false>();
        return true;
    case 615:
        if (args) *err = launch_exact_glynn<38, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 3, true>();
        return true;
    case 646:
        if (args) *err = launch_exact_glynn<40, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 3, false>();
        return true;
    case 663:
        if (args) *err = launch_exact_glynn<41, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 3, true>();
        return true;
    case 694:
        if (args) *err = launch_exact_glynn<43, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 3, false>();
        return true;
    case 711:
        if (args) *err = launch_exact_glynn<44, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 3, true>();
        return true;
    case 742:
        if (args) *err = launch_exact_glynn<46, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 3, false>();
        return true;
    case 759:
        if (args) *err = launch_exact_glynn<47, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 3, true>();
        return true;
    default: return false;
    }
}

}  // namespace pg
