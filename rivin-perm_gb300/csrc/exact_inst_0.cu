// Instantiations of the exact Glynn kernel (part 0 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_0(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 34:
        if (args) *err = launch_exact_glynn<2, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<2, 1, false>();
        return true;
    case 84:
        if (args) *err = launch_exact_glynn<5, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 2, false>();
        return true;
    case 116:
        if (args) *err = launch_exact_glynn<7, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 2, false>();
        return true;
    case 148:
        if (args) *err = launch_exact_glynn<9, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 2, false>();
        return true;
    case 180:
        if (args) *err = launch_exact_glynn<11, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 2, false>();
        return true;
    case 212:
        if (args) *err = launch_exact_glynn<13, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 2, false>();
        return true;
    case 244:
        if (args) *err = launch_exact_glynn<15, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 2, false>();
        return true;
    case 278:
        if (args) *err = launch_exact_glynn<17, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 3, false>();
        return true;
    case 311:
        if (args) *err = launch_exact_glynn<19, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 3, true>();
        return true;
    case 356:
        if (args) *err = launch_exact_glynn<22, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 2, false>();
        return true;
    case 392:
        if (args) *err = launch_exact_glynn<24, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 4, false>();
        return true;
    case 407:
        if (args) *err = launch_exact_glynn<25, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 3, true>();
        return true;
    case 429:
        if (args) *err = launch_exact_glynn<26, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 6, true>();
        return true;
    case 456:
        if (args) *err = launch_exact_glynn<28, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 4, false>();
        return true;
    case 471:
        if (args) *err = launch_exact_glynn<29, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 3, true>();
        return true;
    case 493:
        if (args) *err = launch_exact_glynn<30, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 6, true>();
        return true;
    case 520:
        if (args) *err = launch_exact_glynn<32, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 4, false>();
        return true;
    case 537:
        if (args) *err = launch_exact_glynn<33, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 4, true>();
        return true;
    case 568:
        if (args) *err = launch_exact_glynn<35, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 4, false>();
        return true;
    case 585:
        if (args) *err = launch_exact_glynn<36, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 4, true>();
        return true;
    case 616:
        if (args) *err = launch_exact_glynn<38, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 4, false>();
        return true;
    case 633:
        if (args) *err = launch_exact_glynn<39, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 4, true>();
        return true;
    case 664:
        if (args) *err = launch_exact_glynn<41, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 4, false>();
        return true;
    case 681:
        if (args) *err = launch_exact_glynn<42, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 4, true>();
        return true;
    case 712:
        if (args) *err = launch_exact_glynn<44, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 4, false>();
        return true;
    case 729:
        if (args) *err = launch_exact_glynn<45, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 4, true>();
        return true;
    case 760:
        if (args) *err = launch_exact_glynn<47, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 4, false>();
        return true;
    case 777:
        if (args) *err = launch_exact_glynn<48, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 4, true>();
        return true;
    default: return false;
    }
}

}  // namespace pg
