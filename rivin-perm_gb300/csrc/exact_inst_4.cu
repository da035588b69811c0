// Instantiations of the exact Glynn kernel (part 4 of 6).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_4(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 36:
        if (args) *err = launch_exact_glynn<4, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 4>();
        return true;
    case 60:
        if (args) *err = launch_exact_glynn<7, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 4>();
        return true;
    case 84:
        if (args) *err = launch_exact_glynn<10, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 4>();
        return true;
    case 108:
        if (args) *err = launch_exact_glynn<13, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 4>();
        return true;
    case 132:
        if (args) *err = launch_exact_glynn<16, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 4>();
        return true;
    case 156:
        if (args) *err = launch_exact_glynn<19, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 4>();
        return true;
    case 180:
        if (args) *err = launch_exact_glynn<22, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 4>();
        return true;
    case 198:
        if (args) *err = launch_exact_glynn<24, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 6>();
        return true;
    case 212:
        if (args) *err = launch_exact_glynn<26, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 4>();
        return true;
    case 222:
        if (args) *err = launch_exact_glynn<27, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 6>();
        return true;
    case 236:
        if (args) *err = launch_exact_glynn<29, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 4>();
        return true;
    case 246:
        if (args) *err = launch_exact_glynn<30, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 6>();
        return true;
    case 260:
        if (args) *err = launch_exact_glynn<32, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 4>();
        return true;
    case 270:
        if (args) *err = launch_exact_glynn<33, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 6>();
        return true;
    case 284:
        if (args) *err = launch_exact_glynn<35, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 4>();
        return true;
    case 294:
        if (args) *err = launch_exact_glynn<36, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 6>();
        return true;
    case 308:
        if (args) *err = launch_exact_glynn<38, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 4>();
        return true;
    case 318:
        if (args) *err = launch_exact_glynn<39, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 6>();
        return true;
    case 332:
        if (args) *err = launch_exact_glynn<41, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 4>();
        return true;
    case 342:
        if (args) *err = launch_exact_glynn<42, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 6>();
        return true;
    case 356:
        if (args) *err = launch_exact_glynn<44, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 4>();
        return true;
    case 366:
        if (args) *err = launch_exact_glynn<45, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 6>();
        return true;
    case 380:
        if (args) *err = launch_exact_glynn<47, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 4>();
        return true;
    case 390:
        if (args) *err = launch_exact_glynn<48, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 6>();
        return true;
    default: return false;
    }
}

}  // namespace pg
