// Instantiations of the exact Glynn kernel (part 2 of 8).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_2(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 25:
        if (args) *err = launch_exact_glynn<3, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 1>();
        return true;
    case 42:
        if (args) *err = launch_exact_glynn<5, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 2>();
        return true;
    case 58:
        if (args) *err = launch_exact_glynn<7, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 2>();
        return true;
    case 74:
        if (args) *err = launch_exact_glynn<9, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 2>();
        return true;
    case 90:
        if (args) *err = launch_exact_glynn<11, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 2>();
        return true;
    case 106:
        if (args) *err = launch_exact_glynn<13, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 2>();
        return true;
    case 122:
        if (args) *err = launch_exact_glynn<15, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 2>();
        return true;
    case 139:
        if (args) *err = launch_exact_glynn<17, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 3>();
        return true;
    case 162:
        if (args) *err = launch_exact_glynn<20, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 2>();
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
    case 226:
        if (args) *err = launch_exact_glynn<28, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 2>();
        return true;
    case 237:
        if (args) *err = launch_exact_glynn<29, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 5>();
        return true;
    case 251:
        if (args) *err = launch_exact_glynn<31, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 3>();
        return true;
    case 262:
        if (args) *err = launch_exact_glynn<32, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 6>();
        return true;
    case 278:
        if (args) *err = launch_exact_glynn<34, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 6>();
        return true;
    case 294:
        if (args) *err = launch_exact_glynn<36, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<36, 6>();
        return true;
    case 310:
        if (args) *err = launch_exact_glynn<38, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 6>();
        return true;
    case 326:
        if (args) *err = launch_exact_glynn<40, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 6>();
        return true;
    case 342:
        if (args) *err = launch_exact_glynn<42, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<42, 6>();
        return true;
    case 358:
        if (args) *err = launch_exact_glynn<44, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 6>();
        return true;
    case 374:
        if (args) *err = launch_exact_glynn<46, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 6>();
        return true;
    case 390:
        if (args) *err = launch_exact_glynn<48, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<48, 6>();
        return true;
    default: return false;
    }
}

}  // namespace pg
