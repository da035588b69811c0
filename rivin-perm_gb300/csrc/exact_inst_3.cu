// Instantiations of the exact Glynn kernel (part 3 of 8).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_3(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 26:
        if (args) *err = launch_exact_glynn<3, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 2>();
        return true;
    case 43:
        if (args) *err = launch_exact_glynn<5, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 3>();
        return true;
    case 59:
        if (args) *err = launch_exact_glynn<7, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 3>();
        return true;
    case 75:
        if (args) *err = launch_exact_glynn<9, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 3>();
        return true;
    case 91:
        if (args) *err = launch_exact_glynn<11, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 3>();
        return true;
    case 107:
        if (args) *err = launch_exact_glynn<13, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 3>();
        return true;
    case 123:
        if (args) *err = launch_exact_glynn<15, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 3>();
        return true;
    case 140:
        if (args) *err = launch_exact_glynn<17, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 4>();
        return true;
    case 163:
        if (args) *err = launch_exact_glynn<20, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 3>();
        return true;
    case 186:
        if (args) *err = launch_exact_glynn<23, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 2>();
        return true;
    case 202:
        if (args) *err = launch_exact_glynn<25, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 2>();
        return true;
    case 213:
        if (args) *err = launch_exact_glynn<26, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 5>();
        return true;
    case 227:
        if (args) *err = launch_exact_glynn<28, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 3>();
        return true;
    case 238:
        if (args) *err = launch_exact_glynn<29, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 6>();
        return true;
    case 252:
        if (args) *err = launch_exact_glynn<31, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 4>();
        return true;
    case 267:
        if (args) *err = launch_exact_glynn<33, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 3>();
        return true;
    case 283:
        if (args) *err = launch_exact_glynn<35, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 3>();
        return true;
    case 299:
        if (args) *err = launch_exact_glynn<37, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 3>();
        return true;
    case 315:
        if (args) *err = launch_exact_glynn<39, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 3>();
        return true;
    case 331:
        if (args) *err = launch_exact_glynn<41, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 3>();
        return true;
    case 347:
        if (args) *err = launch_exact_glynn<43, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 3>();
        return true;
    case 363:
        if (args) *err = launch_exact_glynn<45, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 3>();
        return true;
    case 379:
        if (args) *err = launch_exact_glynn<47, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 3>();
        return true;
    default: return false;
    }
}

}  // namespace pg
