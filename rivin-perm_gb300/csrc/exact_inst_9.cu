// Instantiations of the exact Glynn kernel (part 9 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_9(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 71:
        if (args) *err = launch_exact_glynn<4, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 3, true>();
        return true;
    case 103:
        if (args) *err = launch_exact_glynn<6, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 3, true>();
        return true;
    case 135:
        if (args) *err = launch_exact_glynn<8, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 3, true>();
        return true;
    case 167:
        if (args) *err = launch_exact_glynn<10, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 3, true>();
        return true;
    case 199:
        if (args) *err = launch_exact_glynn<12, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 3, true>();
        return true;
    case 231:
        if (args) *err = launch_exact_glynn<14, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 3, true>();
        return true;
    case 263:
        if (args) *err = launch_exact_glynn<16, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 3, true>();
        return true;
    case 308:
        if (args) *err = launch_exact_glynn<19, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 2, false>();
        return true;
    case 344:
        if (args) *err = launch_exact_glynn<21, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 4, false>();
        return true;
    case 377:
        if (args) *err = launch_exact_glynn<23, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 4, true>();
        return true;
    case 408:
        if (args) *err = launch_exact_glynn<25, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 4, false>();
        return true;
    case 423:
        if (args) *err = launch_exact_glynn<26, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 3, true>();
        return true;
    case 445:
        if (args) *err = launch_exact_glynn<27, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 6, true>();
        return true;
    case 472:
        if (args) *err = launch_exact_glynn<29, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 4, false>();
        return true;
    case 487:
        if (args) *err = launch_exact_glynn<30, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 3, true>();
        return true;
    case 509:
        if (args) *err = launch_exact_glynn<31, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 6, true>();
        return true;
    case 538:
        if (args) *err = launch_exact_glynn<33, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 5, false>();
        return true;
    case 555:
        if (args) *err = launch_exact_glynn<34, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 5, true>();
        return true;
    case 586:
        if (args) *err = launch_exact_glynn<36, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 5, false>();
        return true;
    case 603:
        if (args) *err = launch_exact_glynn<37, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 5, true>();
        return true;
    case 634:
        if (args) *err = launch_exact_glynn<39, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 5, false>();
        return true;
    case 651:
        if (args) *err = launch_exact_glynn<40, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 5, true>();
        return true;
    case 682:
        if (args) *err = launch_exact_glynn<42, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 5, false>();
        return true;
    case 699:
        if (args) *err = launch_exact_glynn<43, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 5, true>();
        return true;
    case 730:
        if (args) *err = launch_exact_glynn<45, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 5, false>();
        return true;
    case 747:
        if (args) *err = launch_exact_glynn<46, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 5, true>();
        return true;
    case 778:
        if (args) *err = launch_exact_glynn<48, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 5, false>();
        return true;
    default: return false;
    }
}

}  // namespace pg
