// Instantiations of the exact Glynn kernel (part 5 of 8).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_5(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 33:
        if (args) *err = launch_exact_glynn<4, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<4, 1>();
        return true;
    case 49:
        if (args) *err = launch_exact_glynn<6, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<6, 1>();
        return true;
    case 65:
        if (args) *err = launch_exact_glynn<8, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 1>();
        return true;
    case 81:
        if (args) *err = launch_exact_glynn<10, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<10, 1>();
        return true;
    case 97:
        if (args) *err = launch_exact_glynn<12, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<12, 1>();
        return true;
    case 113:
        if (args) *err = launch_exact_glynn<14, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 1>();
        return true;
    case 129:
        if (args) *err = launch_exact_glynn<16, 1>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<16, 1>();
        return true;
    case 147:
        if (args) *err = launch_exact_glynn<18, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 3>();
        return true;
    case 170:
        if (args) *err = launch_exact_glynn<21, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<21, 2>();
        return true;
    case 188:
        if (args) *err = launch_exact_glynn<23, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 4>();
        return true;
    case 204:
        if (args) *err = launch_exact_glynn<25, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 4>();
        return true;
    case 218:
        if (args) *err = launch_exact_glynn<27, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<27, 2>();
        return true;
    case 229:
        if (args) *err = launch_exact_glynn<28, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 5>();
        return true;
    case 243:
        if (args) *err = launch_exact_glynn<30, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 3>();
        return true;
    case 254:
        if (args) *err = launch_exact_glynn<31, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 6>();
        return true;
    case 269:
        if (args) *err = launch_exact_glynn<33, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 5>();
        return true;
    case 285:
        if (args) *err = launch_exact_glynn<35, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 5>();
        return true;
    case 301:
        if (args) *err = launch_exact_glynn<37, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 5>();
        return true;
    case 317:
        if (args) *err = launch_exact_glynn<39, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 5>();
        return true;
    case 333:
        if (args) *err = launch_exact_glynn<41, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 5>();
        return true;
    case 349:
        if (args) *err = launch_exact_glynn<43, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 5>();
        return true;
    case 365:
        if (args) *err = launch_exact_glynn<45, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 5>();
        return true;
    case 381:
        if (args) *err = launch_exact_glynn<47, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 5>();
        return true;
    default: return false;
    }
}

}  // namespace pg
