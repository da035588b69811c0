// Float-row shapes (order N, group size G, float rows per group FR) of the
// exact Glynn kernel (exact_float_row in exact_glynn.cuh): groups of 4 with
// 3 float rows for small-entry matrices of orders 24..32 (entries in
// [-8, 8]: three row bounds multiply below 2^22).  Larger groups of 0/1
// matrices were measured slower with float rows (groups of 7 with 5 and of
// 10 with 8 at order 40: 20-24 % slower; the kernels spill and the FMUL
// chains are long), and order 36 spills with groups of 4.
#include "exact_glynn.cuh"

namespace pg {

#define PG_EXACT_FROWS_SHAPES(X) X(24, 4, 3) X(28, 4, 3) X(32, 4, 3)

static constexpr int frows_key(int N, int G, int FR) { return (N * 16 + G) * 16 + FR; }

int exact_frows_max(int N, int G) {
    if (!EXACT_FROWS) return 0;
    int best = 0;
#define PG_FR_MAX(NN, GG, FF) if (N == NN && G == GG && FF > best) best = FF;
    PG_EXACT_FROWS_SHAPES(PG_FR_MAX)
#undef PG_FR_MAX
    return best;
}

cudaError_t launch_exact_frows(int N, int G, int FR, const ExactArgs &args, int blocks,
                               cudaStream_t stream) {
    switch (frows_key(N, G, FR)) {
#define PG_FR_LAUNCH(NN, GG, FF) \
    case frows_key(NN, GG, FF): return launch_exact_glynn<NN, GG, FF>(args, blocks, stream);
        PG_EXACT_FROWS_SHAPES(PG_FR_LAUNCH)
#undef PG_FR_LAUNCH
    default:
        return cudaErrorInvalidValue;
    }
}

int occupancy_exact_frows(int N, int G, int FR) {
    switch (frows_key(N, G, FR)) {
#define PG_FR_OCC(NN, GG, FF) case frows_key(NN, GG, FF): return occupancy_exact_glynn<NN, GG, FF>();
        PG_EXACT_FROWS_SHAPES(PG_FR_OCC)
#undef PG_FR_OCC
    default:
        return 1;
    }
}

}  // namespace pg
