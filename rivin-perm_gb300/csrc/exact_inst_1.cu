// Instantiations of the exact Glynn kernel (part 1 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_1(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 36:
        if (args) *err = launch_exact_glynn<2, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<2, 2, false>();
        return true;
    case 86:
        if (args) *err = launch_exact_glynn<5, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 3, false>();
        return true;
    case 118:
        if (args) *err = launch_exact_glynn<7, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 3, false>();
        return true;
    case 150:
        if (args) *err = launch_exact_glynn<9, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 3, false>();
        return true;
    case 182:
        if (args) *err = launch_exact_glynn<11, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 3, false>();
        return true;
    case 214:
        if (args) *err = launch_exact_glynn<13, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 3, false>();
        return true;
    case 246:
        if (args) *err = launch_exact_glynn<15, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 3, false>();
        return true;
    case 280:
        if (args) *err = launch_exact_glynn<17, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 4, false>();
        return true;
    case 313:
        if (args) *err = launch_exact_glynn<19, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 4, true>();
        return true;
    case 358:
        if (args) *err = launch_exact_glynn<22, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 3, false>();
        return true;
    case 394:
        if (args) *err = launch_exact_glynn<24, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 5, false>();
        return true;
    case 409:
        if (args) *err = launch_exact_glynn<25, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 4, true>();
        return true;
    case 436:
        if (args) *err = launch_exact_glynn<27, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 2, false>();
        return true;
    case 458:
        if (args) *err = launch_exact_glynn<28, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 5, false>();
        return true;
    case 473:
        if (args) *err = launch_exact_glynn<29, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 4, true>();
        return true;
    case 500:
        if (args) *err = launch_exact_glynn<31, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 2, false>();
        return true;
    case 522:
        if (args) *err = launch_exact_glynn<32, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 5, false>();
        return true;
    case 539:
        if (args) *err = launch_exact_glynn<33, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 5, true>();
        return true;
    case 570:
        if (args) *err = launch_exact_glynn<35, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 5, false>();
        return true;
    case 587:
        if (args) *err = launch_exact_glynn<36, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 5, true>();
        return true;
    case 618:
        if (args) *err = launch_exact_glynn<38, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 5, false>();
        return true;
    case 635:
        if (args) *err = launch_exact_glynn<39, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 5, true>();
        return true;
    case 666:
        if (args) *err = launch_exact_glynn<41, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 5, false>();
        return true;
    case 683:
        if (args) *err = launch_exact_glynn<42, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 5, true>();
        return true;
    case 714:
        if (args) *err = launch_exact_glynn<44, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 5, false>();
        return true;
    case 731:
        if (args) *err = launch_exact_glynn<45, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 5, true>();
        return true;
    case 762:
        if (args) *err = launch_exact_glynn<47, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 5, false>();
        return true;
    case 779:
        if (args) *err = launch_exact_glynn<48, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 5, true>();
        return true;
    default: return false;
    }
}

}  // namespace pg
