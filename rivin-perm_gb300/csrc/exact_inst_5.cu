// Instantiations of the exact Glynn kernel (part 5 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_5(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 66:
        if (args) *err = launch_exact_glynn<4, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 1, false>();
        return true;
    case 98:
        if (args) *err = launch_exact_glynn<6, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 1, false>();
        return true;
    case 130:
        if (args) *err = launch_exact_glynn<8, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 1, false>();
        return true;
    case 162:
        if (args) *err = launch_exact_glynn<10, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 1, false>();
        return true;
    case 194:
        if (args) *err = launch_exact_glynn<12, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 1, false>();
        return true;
    case 226:
        if (args) *err = launch_exact_glynn<14, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 1, false>();
        return true;
    case 258:
        if (args) *err = launch_exact_glynn<16, 1, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 1, false>();
        return true;
    case 294:
        if (args) *err = launch_exact_glynn<18, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 3, false>();
        return true;
    case 327:
        if (args) *err = launch_exact_glynn<20, 3, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 3, true>();
        return true;
    case 372:
        if (args) *err = launch_exact_glynn<23, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 2, false>();
        return true;
    case 395:
        if (args) *err = launch_exact_glynn<24, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 5, true>();
        return true;
    case 422:
        if (args) *err = launch_exact_glynn<26, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 3, false>();
        return true;
    case 444:
        if (args) *err = launch_exact_glynn<27, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 6, false>();
        return true;
    case 459:
        if (args) *err = launch_exact_glynn<28, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 5, true>();
        return true;
    case 486:
        if (args) *err = launch_exact_glynn<30, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 3, false>();
        return true;
    case 508:
        if (args) *err = launch_exact_glynn<31, 6, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 6, false>();
        return true;
    case 523:
        if (args) *err = launch_exact_glynn<32, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 5, true>();
        return true;
    case 554:
        if (args) *err = launch_exact_glynn<34, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 5, false>();
        return true;
    case 571:
        if (args) *err = launch_exact_glynn<35, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 5, true>();
        return true;
    case 602:
        if (args) *err = launch_exact_glynn<37, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 5, false>();
        return true;
    case 619:
        if (args) *err = launch_exact_glynn<38, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 5, true>();
        return true;
    case 650:
        if (args) *err = launch_exact_glynn<40, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 5, false>();
        return true;
    case 667:
        if (args) *err = launch_exact_glynn<41, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 5, true>();
        return true;
    case 698:
        if (args) *err = launch_exact_glynn<43, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 5, false>();
        return true;
    case 715:
        if (args) *err = launch_exact_glynn<44, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 5, true>();
        return true;
    case 746:
        if (args) *err = launch_exact_glynn<46, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 5, false>();
        return true;
    case 763:
        if (args) *err = launch_exact_glynn<47, 5, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 5, true>();
        return true;
    default: return false;
    }
}

}  // namespace pg
