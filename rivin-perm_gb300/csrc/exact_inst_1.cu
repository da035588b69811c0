// Instantiations of the exact Glynn kernel (part 1 of 8).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_1(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 18:
        if (args) *err = launch_exact_glynn<2, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<2, 2>();
        return true;
    case 41:
        if (args) *err = launch_exact_glynn<5, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 1>();
        return true;
    case 57:
        if (args) *err = launch_exact_glynn<7, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 1>();
        return true;
    case 73:
        if (args) *err = launch_exact_glynn<9, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 1>();
        return true;
    case 89:
        if (args) *err = launch_exact_glynn<11, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 1>();
        return true;
    case 105:
        if (args) *err = launch_exact_glynn<13, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 1>();
        return true;
    case 121:
        if (args) *err = launch_exact_glynn<15, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 1>();
        return true;
    case 138:
        if (args) *err = launch_exact_glynn<17, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 2>();
        return true;
    case 156:
        if (args) *err = launch_exact_glynn<19, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 4>();
        return true;
    case 179:
        if (args) *err = launch_exact_glynn<22, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 3>();
        return true;
    case 197:
        if (args) *err = launch_exact_glynn<24, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 5>();
        return true;
    case 211:
        if (args) *err = launch_exact_glynn<26, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 3>();
        return true;
    case 222:
        if (args) *err = launch_exact_glynn<27, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 6>();
        return true;
    case 236:
        if (args) *err = launch_exact_glynn<29, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 4>();
        return true;
    case 250:
        if (args) *err = launch_exact_glynn<31, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 2>();
        return true;
    case 261:
        if (args) *err = launch_exact_glynn<32, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 5>();
        return true;
    case 277:
        if (args) *err = launch_exact_glynn<34, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 5>();
        return true;
    case 293:
        if (args) *err = launch_exact_glynn<36, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 5>();
        return true;
    case 309:
        if (args) *err = launch_exact_glynn<38, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 5>();
        return true;
    case 325:
        if (args) *err = launch_exact_glynn<40, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 5>();
        return true;
    case 341:
        if (args) *err = launch_exact_glynn<42, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 5>();
        return true;
    case 357:
        if (args) *err = launch_exact_glynn<44, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 5>();
        return true;
    case 373:
        if (args) *err = launch_exact_glynn<46, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 5>();
        return true;
    case 389:
        if (args) *err = launch_exact_glynn<48, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 5>();
        return true;
    default: return false;
    }
}

}  // namespace pg
