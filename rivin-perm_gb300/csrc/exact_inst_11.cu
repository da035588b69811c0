// Instantiations of the exact Glynn kernel (part 11 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_11(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 82:
        if (args) *err = launch_exact_glynn<5, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 1, false>();
        return true;
    case 114:
        if (args) *err = launch_exact_glynn<7, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 1, false>();
        return true;
    case 146:
        if (args) *err = launch_exact_glynn<9, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 1, false>();
        return true;
    case 178:
        if (args) *err = launch_exact_glynn<11, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 1, false>();
        return true;
    case 210:
        if (args) *err = launch_exact_glynn<13, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 1, false>();
        return true;
    case 242:
        if (args) *err = launch_exact_glynn<15, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 1, false>();
        return true;
    case 276:
        if (args) *err = launch_exact_glynn<17, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 2, false>();
        return true;
    case 312:
        if (args) *err = launch_exact_glynn<19, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 4, false>();
        return true;
    case 345:
        if (args) *err = launch_exact_glynn<21, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 4, true>();
        return true;
    case 390:
        if (args) *err = launch_exact_glynn<24, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 3, false>();
        return true;
    case 412:
        if (args) *err = launch_exact_glynn<25, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 6, false>();
        return true;
    case 427:
        if (args) *err = launch_exact_glynn<26, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 5, true>();
        return true;
    case 454:
        if (args) *err = launch_exact_glynn<28, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 3, false>();
        return true;
    case 476:
        if (args) *err = launch_exact_glynn<29, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 6, false>();
        return true;
    case 491:
        if (args) *err = launch_exact_glynn<30, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 5, true>();
        return true;
    case 518:
        if (args) *err = launch_exact_glynn<32, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 3, false>();
        return true;
    case 535:
        if (args) *err = launch_exact_glynn<33, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 3, true>();
        return true;
    case 566:
        if (args) *err = launch_exact_glynn<35, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 3, false>();
        return true;
    case 583:
        if (args) *err = launch_exact_glynn<36, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 3, true>();
        return true;
    case 614:
        if (args) *err = launch_exact_glynn<38, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 3, false>();
        return true;
    case 631:
        if (args) *err = launch_exact_glynn<39, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 3, true>();
        return true;
    case 662:
        if (args) *err = launch_exact_glynn<41, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 3, false>();
        return true;
    case 679:
        if (args) *err = launch_exact_glynn<42, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 3, true>();
        return true;
    case 710:
        if (args) *err = launch_exact_glynn<44, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 3, false>();
        return true;
    case 727:
        if (args) *err = launch_exact_glynn<45, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 3, true>();
        return true;
    case 758:
        if (args) *err = launch_exact_glynn<47, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 3, false>();
        return true;
    case 775:
        if (args) *err = launch_exact_glynn<48, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 3, true>();
        return true;
    default: return false;
    }
}

}  // namespace pg
