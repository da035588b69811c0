// Instantiations of the exact Glynn kernel (part 10 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_10(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 73:
        if (args) *err = launch_exact_glynn<4, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 4, true>();
        return true;
    case 105:
        if (args) *err = launch_exact_glynn<6, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 4, true>();
        return true;
    case 137:
        if (args) *err = launch_exact_glynn<8, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 4, true>();
        return true;
    case 169:
        if (args) *err = launch_exact_glynn<10, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 4, true>();
        return true;
    case 201:
        if (args) *err = launch_exact_glynn<12, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 4, true>();
        return true;
    case 233:
        if (args) *err = launch_exact_glynn<14, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 4, true>();
        return true;
    case 265:
        if (args) *err = launch_exact_glynn<16, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 4, true>();
        return true;
    case 310:
        if (args) *err = launch_exact_glynn<19, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 3, false>();
        return true;
    case 343:
        if (args) *err = launch_exact_glynn<21, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 3, true>();
        return true;
    case 388:
        if (args) *err = launch_exact_glynn<24, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 2, false>();
        return true;
    case 410:
        if (args) *err = launch_exact_glynn<25, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 5, false>();
        return true;
    case 425:
        if (args) *err = launch_exact_glynn<26, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 4, true>();
        return true;
    case 452:
        if (args) *err = launch_exact_glynn<28, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 2, false>();
        return true;
    case 474:
        if (args) *err = launch_exact_glynn<29, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 5, false>();
        return true;
    case 489:
        if (args) *err = launch_exact_glynn<30, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 4, true>();
        return true;
    case 516:
        if (args) *err = launch_exact_glynn<32, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 2, false>();
        return true;
    case 540:
        if (args) *err = launch_exact_glynn<33, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 6, false>();
        return true;
    case 557:
        if (args) *err = launch_exact_glynn<34, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 6, true>();
        return true;
    case 588:
        if (args) *err = launch_exact_glynn<36, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 6, false>();
        return true;
    case 605:
        if (args) *err = launch_exact_glynn<37, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 6, true>();
        return true;
    case 636:
        if (args) *err = launch_exact_glynn<39, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 6, false>();
        return true;
    case 653:
        if (args) *err = launch_exact_glynn<40, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 6, true>();
        return true;
    case 684:
        if (args) *err = launch_exact_glynn<42, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 6, false>();
        return true;
    case 701:
        if (args) *err = launch_exact_glynn<43, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 6, true>();
        return true;
    case 732:
        if (args) *err = launch_exact_glynn<45, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 6, false>();
        return true;
    case 749:
        if (args) *err = launch_exact_glynn<46, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 6, true>();
        return true;
    case 780:
        if (args) *err = launch_exact_glynn<48, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 6, false>();
        return true;
    default: return false;
    }
}

}  // namespace pg
