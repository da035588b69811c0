// Instantiations of the exact Glynn kernel (part 3 of 6).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_3(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 35:
        if (args) *err = launch_exact_glynn<4, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 3>();
        return true;
    case 59:
        if (args) *err = launch_exact_glynn<7, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 3>();
        return true;
    case 83:
        if (args) *err = launch_exact_glynn<10, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 3>();
        return true;
    case 107:
        if (args) *err = launch_exact_glynn<13, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 3>();
        return true;
    case 131:
        if (args) *err = launch_exact_glynn<16, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 3>();
        return true;
    case 155:
        if (args) *err = launch_exact_glynn<19, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 3>();
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
    case 221:
        if (args) *err = launch_exact_glynn<27, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 5>();
        return true;
    case 235:
        if (args) *err = launch_exact_glynn<29, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 3>();
        return true;
    case 245:
        if (args) *err = launch_exact_glynn<30, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 5>();
        return true;
    case 259:
        if (args) *err = launch_exact_glynn<32, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 3>();
        return true;
    case 269:
        if (args) *err = launch_exact_glynn<33, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 5>();
        return true;
    case 283:
        if (args) *err = launch_exact_glynn<35, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 3>();
        return true;
    case 293:
        if (args) *err = launch_exact_glynn<36, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 5>();
        return true;
    case 307:
        if (args) *err = launch_exact_glynn<38, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 3>();
        return true;
    case 317:
        if (args) *err = launch_exact_glynn<39, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 5>();
        return true;
    case 331:
        if (args) *err = launch_exact_glynn<41, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 3>();
        return true;
    case 341:
        if (args) *err = launch_exact_glynn<42, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 5>();
        return true;
    case 355:
        if (args) *err = launch_exact_glynn<44, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 3>();
        return true;
    case 365:
        if (args) *err = launch_exact_glynn<45, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 5>();
        return true;
    case 379:
        if (args) *err = launch_exact_glynn<47, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 3>();
        return true;
    case 389:
        if (args) *err = launch_exact_glynn<48, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 5>();
        return true;
    default: return false;
    }
}

}  // namespace pg
