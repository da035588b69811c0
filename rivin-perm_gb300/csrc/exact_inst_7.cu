// Instantiations of the exact Glynn kernel (part 7 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_7(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 70:
        if (args) *err = launch_exact_glynn<4, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 3, false>();
        return true;
    case 102:
        if (args) *err = launch_exact_glynn<6, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 3, false>();
        return true;
    case 134:
        if (args) *err = launch_exact_glynn<8, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 3, false>();
        return true;
    case 166:
        if (args) *err = launch_exact_glynn<10, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 3, false>();
        return true;
    case 198:
        if (args) *err = launch_exact_glynn<12, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 3, false>();
        return true;
    case 230:
        if (args) *err = launch_exact_glynn<14, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 3, false>();
        return true;
    case 262:
        if (args) *err = launch_exact_glynn<16, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 3, false>();
        return true;
    case 295:
        if (args) *err = launch_exact_glynn<18, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 3, true>();
        return true;
    case 340:
        if (args) *err = launch_exact_glynn<21, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 2, false>();
        return true;
    case 376:
        if (args) *err = launch_exact_glynn<23, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 4, false>();
        return true;
    case 404:
        if (args) *err = launch_exact_glynn<25, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 2, false>();
        return true;
    case 426:
        if (args) *err = launch_exact_glynn<26, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 5, false>();
        return true;
    case 441:
        if (args) *err = launch_exact_glynn<27, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 4, true>();
        return true;
    case 468:
        if (args) *err = launch_exact_glynn<29, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 2, false>();
        return true;
    case 490:
        if (args) *err = launch_exact_glynn<30, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 5, false>();
        return true;
    case 505:
        if (args) *err = launch_exact_glynn<31, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 4, true>();
        return true;
    case 534:
        if (args) *err = launch_exact_glynn<33, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 3, false>();
        return true;
    case 551:
        if (args) *err = launch_exact_glynn<34, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 3, true>();
        return true;
    case 582:
        if (args) *err = launch_exact_glynn<36, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 3, false>();
        return true;
    case 599:
        if (args) *err = launch_exact_glynn<37, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 3, true>();
        return true;
    case 630:
        if (args) *err = launch_exact_glynn<39, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 3, false>();
        return true;
    case 647:
        if (args) *err = launch_exact_glynn<40, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 3, true>();
        return true;
    case 678:
        if (args) *err = launch_exact_glynn<42, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 3, false>();
        return true;
    case 695:
        if (args) *err = launch_exact_glynn<43, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 3, true>();
        return true;
    case 726:
        if (args) *err = launch_exact_glynn<45, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 3, false>();
        return true;
    case 743:
        if (args) *err = launch_exact_glynn<46, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 3, true>();
        return true;
    case 774:
        if (args) *err = launch_exact_glynn<48, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 3, false>();
        return true;
    default: return false;
    }
}

}  // namespace pg
