// Instantiations of the exact Glynn kernel (part 1 of 6).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_1(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 26:
        if (args) *err = launch_exact_glynn<3, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 2>();
        return true;
    case 51:
        if (args) *err = launch_exact_glynn<6, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 3>();
        return true;
    case 75:
        if (args) *err = launch_exact_glynn<9, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 3>();
        return true;
    case 99:
        if (args) *err = launch_exact_glynn<12, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 3>();
        return true;
    case 123:
        if (args) *err = launch_exact_glynn<15, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 3>();
        return true;
    case 147:
        if (args) *err = launch_exact_glynn<18, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 3>();
        return true;
    case 171:
        if (args) *err = launch_exact_glynn<21, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 3>();
        return true;
    case 195:
        if (args) *err = launch_exact_glynn<24, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 3>();
        return true;
    case 205:
        if (args) *err = launch_exact_glynn<25, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 5>();
        return true;
    case 219:
        if (args) *err = launch_exact_glynn<27, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 3>();
        return true;
    case 229:
        if (args) *err = launch_exact_glynn<28, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 5>();
        return true;
    case 243:
        if (args) *err = launch_exact_glynn<30, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 3>();
        return true;
    case 253:
        if (args) *err = launch_exact_glynn<31, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 5>();
        return true;
    case 267:
        if (args) *err = launch_exact_glynn<33, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 3>();
        return true;
    case 277:
        if (args) *err = launch_exact_glynn<34, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 5>();
        return true;
    case 291:
        if (args) *err = launch_exact_glynn<36, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 3>();
        return true;
    case 301:
        if (args) *err = launch_exact_glynn<37, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 5>();
        return true;
    case 315:
        if (args) *err = launch_exact_glynn<39, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 3>();
        return true;
    case 325:
        if (args) *err = launch_exact_glynn<40, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 5>();
        return true;
    case 339:
        if (args) *err = launch_exact_glynn<42, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 3>();
        return true;
    case 349:
        if (args) *err = launch_exact_glynn<43, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 5>();
        return true;
    case 363:
        if (args) *err = launch_exact_glynn<45, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 3>();
        return true;
    case 373:
        if (args) *err = launch_exact_glynn<46, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 5>();
        return true;
    case 387:
        if (args) *err = launch_exact_glynn<48, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 3>();
        return true;
    default: return false;
    }
}

}  // namespace pg
