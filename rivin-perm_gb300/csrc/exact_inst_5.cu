// Instantiations of the exact Glynn kernel (part 5 of 6).
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_5(int N, int G, const ExactArgs *args, int blocks,
                       cudaStream_t stream, cudaError_t *err, int *occ) {
    switch (N * 8 + G) {
    case 43:
        if (args) *err = launch_exact_glynn<5, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<5, 3>();
        return true;
    case 67:
        if (args) *err = launch_exact_glynn<8, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<8, 3>();
        return true;
    case 91:
        if (args) *err = launch_exact_glynn<11, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<11, 3>();
        return true;
    case 115:
        if (args) *err = launch_exact_glynn<14, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<14, 3>();
        return true;
    case 139:
        if (args) *err = launch_exact_glynn<17, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<17, 3>();
        return true;
    case 163:
        if (args) *err = launch_exact_glynn<20, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<20, 3>();
        return true;
    case 187:
        if (args) *err = launch_exact_glynn<23, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<23, 3>();
        return true;
    case 203:
        if (args) *err = launch_exact_glynn<25, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<25, 3>();
        return true;
    case 213:
        if (args) *err = launch_exact_glynn<26, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<26, 5>();
        return true;
    case 227:
        if (args) *err = launch_exact_glynn<28, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<28, 3>();
        return true;
    case 237:
        if (args) *err = launch_exact_glynn<29, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<29, 5>();
        return true;
    case 251:
        if (args) *err = launch_exact_glynn<31, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<31, 3>();
        return true;
    case 261:
        if (args) *err = launch_exact_glynn<32, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<32, 5>();
        return true;
    case 275:
        if (args) *err = launch_exact_glynn<34, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<34, 3>();
        return true;
    case 285:
        if (args) *err = launch_exact_glynn<35, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<35, 5>();
        return true;
    case 299:
        if (args) *err = launch_exact_glynn<37, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<37, 3>();
        return true;
    case 309:
        if (args) *err = launch_exact_glynn<38, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<38, 5>();
        return true;
    case 323:
        if (args) *err = launch_exact_glynn<40, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<40, 3>();
        return true;
    case 333:
        if (args) *err = launch_exact_glynn<41, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<41, 5>();
        return true;
    case 347:
        if (args) *err = launch_exact_glynn<43, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<43, 3>();
        return true;
    case 357:
        if (args) *err = launch_exact_glynn<44, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<44, 5>();
        return true;
    case 371:
        if (args) *err = launch_exact_glynn<46, 3>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<46, 3>();
        return true;
    case 381:
        if (args) *err = launch_exact_glynn<47, 5>(*args, blocks, stream);
        if (occ) *occ = occupancy_exact_glynn<47, 5>();
        return true;
    default: return false;
    }
}

}  // namespace pg
