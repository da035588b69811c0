// Instantiations of the exact Glynn kernel (part 6 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_6(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 68:
        if (args) *err = launch_exact_glynn<4, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 2, false>();
        return true;
    case 100:
        if (args) *err = launch_exact_glynn<6, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 2, false>();
        return true;
    case 132:
        if (args) *err = launch_exact_glynn<8, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 2, false>();
        return true;
    case 164:
        if (args) *err = launch_exact_glynn<10, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 2, false>();
        return true;
    case 196:
        if (args) *err = launch_exact_glynn<12, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 2, false>();
        return true;
    case 228:
        if (args) *err = launch_exact_glynn<14, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 2, false>();
        return true;
    case 260:
        if (args) *err = launch_exact_glynn<16, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 2, false>();
        return true;
    case 296:
        if (args) *err = launch_exact_glynn<18, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 4, false>();
        return true;
    case 329:
        if (args) *err = launch_exact_glynn<20, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 4, true>();
        return true;
    case 374:
        if (args) *err = launch_exact_glynn<23, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 3, false>();
        return true;
    case 397:
        if (args) *err = launch_exact_glynn<24, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 6, true>();
        return true;
    case 424:
        if (args) *err = launch_exact_glynn<26, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 4, false>();
        return true;
    case 439:
        if (args) *err = launch_exact_glynn<27, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 3, true>();
        return true;
    case 461:
        if (args) *err = launch_exact_glynn<28, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 6, true>();
        return true;
    case 488:
        if (args) *err = launch_exact_glynn<30, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 4, false>();
        return true;
    case 503:
        if (args) *err = launch_exact_glynn<31, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 3, true>();
        return true;
    case 525:
        if (args) *err = launch_exact_glynn<32, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 6, true>();
        return true;
    case 556:
        if (args) *err = launch_exact_glynn<34, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 6, false>();
        return true;
    case 573:
        if (args) *err = launch_exact_glynn<35, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 6, true>();
        return true;
    case 604:
        if (args) *err = launch_exact_glynn<37, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 6, false>();
        return true;
    case 621:
        if (args) *err = launch_exact_glynn<38, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 6, true>();
        return true;
    case 652:
        if (args) *err = launch_exact_glynn<40, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 6, false>();
        return true;
    case 669:
        if (args) *err = launch_exact_glynn<41, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 6, true>();
        return true;
    case 700:
        if (args) *err = launch_exact_glynn<43, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 6, false>();
        return true;
    case 717:
        if (args) *err = launch_exact_glynn<44, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 6, true>();
        return true;
    case 748:
        if (args) *err = launch_exact_glynn<46, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 6, false>();
        return true;
    case 765:
        if (args) *err = launch_exact_glynn<47, 6, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 6, true>();
        return true;
    default: return false;
    }
}

}  // namespace pg
