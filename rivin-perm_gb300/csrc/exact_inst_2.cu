// Instantiations of the exact Glynn kernel (part 2 of 6).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_2(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 27:
        if (args) *err = launch_exact_glynn<3, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 3>();
        return true;
    case 52:
        if (args) *err = launch_exact_glynn<6, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 4>();
        return true;
    case 76:
        if (args) *err = launch_exact_glynn<9, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 4>();
        return true;
    case 100:
        if (args) *err = launch_exact_glynn<12, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 4>();
        return true;
    case 124:
        if (args) *err = launch_exact_glynn<15, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 4>();
        return true;
    case 148:
        if (args) *err = launch_exact_glynn<18, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 4>();
        return true;
    case 172:
        if (args) *err = launch_exact_glynn<21, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 4>();
        return true;
    case 196:
        if (args) *err = launch_exact_glynn<24, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<24, 4>();
        return true;
    case 206:
        if (args) *err = launch_exact_glynn<25, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 6>();
        return true;
    case 220:
        if (args) *err = launch_exact_glynn<27, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 4>();
        return true;
    case 230:
        if (args) *err = launch_exact_glynn<28, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 6>();
        return true;
    case 244:
        if (args) *err = launch_exact_glynn<30, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 4>();
        return true;
    case 254:
        if (args) *err = launch_exact_glynn<31, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 6>();
        return true;
    case 268:
        if (args) *err = launch_exact_glynn<33, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 4>();
        return true;
    case 278:
        if (args) *err = launch_exact_glynn<34, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 6>();
        return true;
    case 292:
        if (args) *err = launch_exact_glynn<36, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 4>();
        return true;
    case 302:
        if (args) *err = launch_exact_glynn<37, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 6>();
        return true;
    case 316:
        if (args) *err = launch_exact_glynn<39, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 4>();
        return true;
    case 326:
        if (args) *err = launch_exact_glynn<40, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 6>();
        return true;
    case 340:
        if (args) *err = launch_exact_glynn<42, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 4>();
        return true;
    case 350:
        if (args) *err = launch_exact_glynn<43, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 6>();
        return true;
    case 364:
        if (args) *err = launch_exact_glynn<45, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 4>();
        return true;
    case 374:
        if (args) *err = launch_exact_glynn<46, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 6>();
        return true;
    case 388:
        if (args) *err = launch_exact_glynn<48, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 4>();
        return true;
    default: return false;
    }
}

}  // namespace pg
