// Instantiations of the exact Glynn kernel (part 4 of 8).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_4(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 27:
        if (args) *err = launch_exact_glynn<3, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<3, 3>();
        return true;
    case 44:
        if (args) *err = launch_exact_glynn<5, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 4>();
        return true;
    case 60:
        if (args) *err = launch_exact_glynn<7, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<7, 4>();
        return true;
    case 76:
        if (args) *err = launch_exact_glynn<9, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<9, 4>();
        return true;
    case 92:
        if (args) *err = launch_exact_glynn<11, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 4>();
        return true;
    case 108:
        if (args) *err = launch_exact_glynn<13, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<13, 4>();
        return true;
    case 124:
        if (args) *err = launch_exact_glynn<15, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<15, 4>();
        return true;
    case 146:
        if (args) *err = launch_exact_glynn<18, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<18, 2>();
        return true;
    case 164:
        if (args) *err = launch_exact_glynn<20, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 4>();
        return true;
    case 187:
        if (args) *err = launch_exact_glynn<23, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 3>();
        return true;
    case 203:
        if (args) *err = launch_exact_glynn<25, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 3>();
        return true;
    case 214:
        if (args) *err = launch_exact_glynn<26, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 6>();
        return true;
    case 228:
        if (args) *err = launch_exact_glynn<28, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 4>();
        return true;
    case 242:
        if (args) *err = launch_exact_glynn<30, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<30, 2>();
        return true;
    case 253:
        if (args) *err = launch_exact_glynn<31, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 5>();
        return true;
    case 268:
        if (args) *err = launch_exact_glynn<33, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<33, 4>();
        return true;
    case 284:
        if (args) *err = launch_exact_glynn<35, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 4>();
        return true;
    case 300:
        if (args) *err = launch_exact_glynn<37, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 4>();
        return true;
    case 316:
        if (args) *err = launch_exact_glynn<39, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<39, 4>();
        return true;
    case 332:
        if (args) *err = launch_exact_glynn<41, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 4>();
        return true;
    case 348:
        if (args) *err = launch_exact_glynn<43, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 4>();
        return true;
    case 364:
        if (args) *err = launch_exact_glynn<45, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<45, 4>();
        return true;
    case 380:
        if (args) *err = launch_exact_glynn<47, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 4>();
        return true;
    default: return false;
    }
}

}  // namespace pg
