// Instantiations of the exact Glynn kernel (part 2 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_2(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 50:
        if (args) *err = launch_exact_glynn<3, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 1, false>();
        return true;
    case 88:
        if (args) *err = launch_exact_glynn<5, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 4, false>();
        return true;
    case 120:
        if (args) *err = launch_exact_glynn<7, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 4, false>();
        return true;
    case 152:
        if (args) *err = launch_exact_glynn<9, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 4, false>();
        return true;
    case 184:
        if (args) *err = launch_exact_glynn<11, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 4, false>();
        return true;
    case 216:
        if (args) *err = launch_exact_glynn<13, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 4, false>();
        return true;
    case 248:
        if (args) *err = launch_exact_glynn<15, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 4, false>();
        return true;
    case 279:
        if (args) *err = launch_exact_glynn<17, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 3, true>();
        return true;
    case 324:
        if (args) *err = launch_exact_glynn<20, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 2, false>();
        return true;
    case 360:
        if (args) *err = launch_exact_glynn<22, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 4, false>();
        return true;
    case 396:
        if (args) *err = launch_exact_glynn<24, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 6, false>();
        return true;
    case 411:
        if (args) *err = launch_exact_glynn<25, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 5, true>();
        return true;
    case 438:
        if (args) *err = launch_exact_glynn<27, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 3, false>();
        return true;
    case 460:
        if (args) *err = launch_exact_glynn<28, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 6, false>();
        return true;
    case 475:
        if (args) *err = launch_exact_glynn<29, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 5, true>();
        return true;
    case 502:
        if (args) *err = launch_exact_glynn<31, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 3, false>();
        return true;
    case 524:
        if (args) *err = launch_exact_glynn<32, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 6, false>();
        return true;
    case 541:
        if (args) *err = launch_exact_glynn<33, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 6, true>();
        return true;
    case 572:
        if (args) *err = launch_exact_glynn<35, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 6, false>();
        return true;
    case 589:
        if (args) *err = launch_exact_glynn<36, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 6, true>();
        return true;
    case 620:
        if (args) *err = launch_exact_glynn<38, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 6, false>();
        return true;
    case 637:
        if (args) *err = launch_exact_glynn<39, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 6, true>();
        return true;
    case 668:
        if (args) *err = launch_exact_glynn<41, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 6, false>();
        return true;
    case 685:
        if (args) *err = launch_exact_glynn<42, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 6, true>();
        return true;
    case 716:
        if (args) *err = launch_exact_glynn<44, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 6, false>();
        return true;
    case 733:
        if (args) *err = launch_exact_glynn<45, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 6, true>();
        return true;
    case 764:
        if (args) *err = launch_exact_glynn<47, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 6, false>();
        return true;
    case 781:
        if (args) *err = launch_exact_glynn<48, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 6, true>();
        return true;
    default: return false;
    }
}

}  // namespace pg
