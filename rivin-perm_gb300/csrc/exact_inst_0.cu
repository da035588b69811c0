// Instantiations of the exact Glynn kernel (part 0 of 8).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_0(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 17:
        if (args) *err = launch_exact_glynn<2, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<2, 1>();
        return true;
    case 36:
        if (args) *err = launch_exact_glynn<4, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 4>();
        return true;
    case 52:
        if (args) *err = launch_exact_glynn<6, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 4>();
        return true;
    case 68:
        if (args) *err = launch_exact_glynn<8, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 4>();
        return true;
    case 84:
        if (args) *err = launch_exact_glynn<10, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 4>();
        return true;
    case 100:
        if (args) *err = launch_exact_glynn<12, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 4>();
        return true;
    case 116:
        if (args) *err = launch_exact_glynn<14, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 4>();
        return true;
    case 132:
        if (args) *err = launch_exact_glynn<16, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 4>();
        return true;
    case 155:
        if (args) *err = launch_exact_glynn<19, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<19, 3>();
        return true;
    case 178:
        if (args) *err = launch_exact_glynn<22, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<22, 2>();
        return true;
    case 196:
        if (args) *err = launch_exact_glynn<24, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 4>();
        return true;
    case 210:
        if (args) *err = launch_exact_glynn<26, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 2>();
        return true;
    case 221:
        if (args) *err = launch_exact_glynn<27, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 5>();
        return true;
    case 235:
        if (args) *err = launch_exact_glynn<29, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 3>();
        return true;
    case 246:
        if (args) *err = launch_exact_glynn<30, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 6>();
        return true;
    case 260:
        if (args) *err = launch_exact_glynn<32, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 4>();
        return true;
    case 276:
        if (args) *err = launch_exact_glynn<34, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 4>();
        return true;
    case 292:
        if (args) *err = launch_exact_glynn<36, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 4>();
        return true;
    case 308:
        if (args) *err = launch_exact_glynn<38, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 4>();
        return true;
    case 324:
        if (args) *err = launch_exact_glynn<40, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 4>();
        return true;
    case 340:
        if (args) *err = launch_exact_glynn<42, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 4>();
        return true;
    case 356:
        if (args) *err = launch_exact_glynn<44, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 4>();
        return true;
    case 372:
        if (args) *err = launch_exact_glynn<46, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 4>();
        return true;
    case 388:
        if (args) *err = launch_exact_glynn<48, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 4>();
        return true;
    default: return false;
    }
}

}  // namespace pg
