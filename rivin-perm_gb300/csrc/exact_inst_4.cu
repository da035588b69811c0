// Instantiations of the exact Glynn kernel (part 4 of 12).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_4(int key, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (key) {
    case 54:
        if (args) *err = launch_exact_glynn<3, 3, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 3, false>();
        return true;
    case 89:
        if (args) *err = launch_exact_glynn<5, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 4, true>();
        return true;
    case 121:
        if (args) *err = launch_exact_glynn<7, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 4, true>();
        return true;
    case 153:
        if (args) *err = launch_exact_glynn<9, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 4, true>();
        return true;
    case 185:
        if (args) *err = launch_exact_glynn<11, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 4, true>();
        return true;
    case 217:
        if (args) *err = launch_exact_glynn<13, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 4, true>();
        return true;
    case 249:
        if (args) *err = launch_exact_glynn<15, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 4, true>();
        return true;
    case 292:
        if (args) *err = launch_exact_glynn<18, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 2, false>();
        return true;
    case 328:
        if (args) *err = launch_exact_glynn<20, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 4, false>();
        return true;
    case 361:
        if (args) *err = launch_exact_glynn<22, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 4, true>();
        return true;
    case 393:
        if (args) *err = launch_exact_glynn<24, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 4, true>();
        return true;
    case 420:
        if (args) *err = launch_exact_glynn<26, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 2, false>();
        return true;
    case 442:
        if (args) *err = launch_exact_glynn<27, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 5, false>();
        return true;
    case 457:
        if (args) *err = launch_exact_glynn<28, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 4, true>();
        return true;
    case 484:
        if (args) *err = launch_exact_glynn<30, 2, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 2, false>();
        return true;
    case 506:
        if (args) *err = launch_exact_glynn<31, 5, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 5, false>();
        return true;
    case 521:
        if (args) *err = launch_exact_glynn<32, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 4, true>();
        return true;
    case 552:
        if (args) *err = launch_exact_glynn<34, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 4, false>();
        return true;
    case 569:
        if (args) *err = launch_exact_glynn<35, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 4, true>();
        return true;
    case 600:
        if (args) *err = launch_exact_glynn<37, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 4, false>();
        return true;
    case 617:
        if (args) *err = launch_exact_glynn<38, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 4, true>();
        return true;
    case 648:
        if (args) *err = launch_exact_glynn<40, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 4, false>();
        return true;
    case 665:
        if (args) *err = launch_exact_glynn<41, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 4, true>();
        return true;
    case 696:
        if (args) *err = launch_exact_glynn<43, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 4, false>();
        return true;
    case 713:
        if (args) *err = launch_exact_glynn<44, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 4, true>();
        return true;
    case 744:
        if (args) *err = launch_exact_glynn<46, 4, false>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 4, false>();
        return true;
    case 761:
        if (args) *err = launch_exact_glynn<47, 4, true>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 4, true>();
        return true;
    default: return false;
    }
}

}  // namespace pg
