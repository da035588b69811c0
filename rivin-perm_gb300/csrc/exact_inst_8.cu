// Instantiations of the exact Glynn kernel (part 8 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_8(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 72:
        if (args) *err = launch_exact_glynn<4, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 4, false>();
        return true;
    case 104:
        if (args) *err = launch_exact_glynn<6, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 4, false>();
        return true;
    case 136:
        if (args) *err = launch_exact_glynn<8, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 4, false>();
        return true;
    case 168:
        if (args) *err = launch_exact_glynn<10, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 4, false>();
        return true;
    case 200:
        if (args) *err = launch_exact_glynn<12, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 4, false>();
        return true;
    case 232:
        if (args) *err = launch_exact_glynn<14, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 4, false>();
        return true;
    case 264:
        if (args) *err = launch_exact_glynn<16, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 4, false>();
        return true;
    case 297:
        if (args) *err = launch_exact_glynn<18, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 4, true>();
        return true;
    case 342:
        if (args) *err = launch_exact_glynn<21, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 3, false>();
        return true;
    case 375:
        if (args) *err = launch_exact_glynn<23, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 3, true>();
        return true;
    case 406:
        if (args) *err = launch_exact_glynn<25, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 3, false>();
        return true;
    case 428:
        if (args) *err = launch_exact_glynn<26, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 6, false>();
        return true;
    case 443:
        if (args) *err = launch_exact_glynn<27, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 5, true>();
        return true;
    case 470:
        if (args) *err = launch_exact_glynn<29, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 3, false>();
        return true;
    case 492:
        if (args) *err = launch_exact_glynn<30, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 6, false>();
        return true;
    case 507:
        if (args) *err = launch_exact_glynn<31, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 5, true>();
        return true;
    case 536:
        if (args) *err = launch_exact_glynn<33, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 4, false>();
        return true;
    case 553:
        if (args) *err = launch_exact_glynn<34, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 4, true>();
        return true;
    case 584:
        if (args) *err = launch_exact_glynn<36, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 4, false>();
        return true;
    case 601:
        if (args) *err = launch_exact_glynn<37, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 4, true>();
        return true;
    case 632:
        if (args) *err = launch_exact_glynn<39, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 4, false>();
        return true;
    case 649:
        if (args) *err = launch_exact_glynn<40, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 4, true>();
        return true;
    case 680:
        if (args) *err = launch_exact_glynn<42, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 4, false>();
        return true;
    case 697:
        if (args) *err = launch_exact_glynn<43, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 4, true>();
        return true;
    case 728:
        if (args) *err = launch_exact_glynn<45, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 4, false>();
        return true;
    case 745:
        if (args) *err = launch_exact_glynn<46, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 4, true>();
        return true;
    case 776:
        if (args) *err = launch_exact_glynn<48, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 4, false>();
        return true;
    default: return false;
    }
}

}  // namespace pg
