// Instantiations of the exact Glynn kernel (part 0 of 6).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_0(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 18:
        if (args) *err = launch_exact_glynn<2, 2>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<2, 2>();
        return true;
    case 44:
        if (args) *err = launch_exact_glynn<5, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 4>();
        return true;
    case 68:
        if (args) *err = launch_exact_glynn<8, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 4>();
        return true;
    case 92:
        if (args) *err = launch_exact_glynn<11, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 4>();
        return true;
    case 116:
        if (args) *err = launch_exact_glynn<14, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 4>();
        return true;
    case 140:
        if (args) *err = launch_exact_glynn<17, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 4>();
        return true;
    case 164:
        if (args) *err = launch_exact_glynn<20, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 4>();
        return true;
    case 188:
        if (args) *err = launch_exact_glynn<23, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 4>();
        return true;
    case 204:
        if (args) *err = launch_exact_glynn<25, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 4>();
        return true;
    case 214:
        if (args) *err = launch_exact_glynn<26, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 6>();
        return true;
    case 228:
        if (args) *err = launch_exact_glynn<28, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 4>();
        return true;
    case 238:
        if (args) *err = launch_exact_glynn<29, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 6>();
        return true;
    case 252:
        if (args) *err = launch_exact_glynn<31, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 4>();
        return true;
    case 262:
        if (args) *err = launch_exact_glynn<32, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 6>();
        return true;
    case 276:
        if (args) *err = launch_exact_glynn<34, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 4>();
        return true;
    case 286:
        if (args) *err = launch_exact_glynn<35, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 6>();
        return true;
    case 300:
        if (args) *err = launch_exact_glynn<37, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 4>();
        return true;
    case 310:
        if (args) *err = launch_exact_glynn<38, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 6>();
        return true;
    case 324:
        if (args) *err = launch_exact_glynn<40, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 4>();
        return true;
    case 334:
        if (args) *err = launch_exact_glynn<41, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 6>();
        return true;
    case 348:
        if (args) *err = launch_exact_glynn<43, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 4>();
        return true;
    case 358:
        if (args) *err = launch_exact_glynn<44, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 6>();
        return true;
    case 372:
        if (args) *err = launch_exact_glynn<46, 4>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 4>();
        return true;
    case 382:
        if (args) *err = launch_exact_glynn<47, 6>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 6>();
        return true;
    default: return false;
    }
}

}  // namespace pg
