// Instantiations of binary_glynn_kernel with 40 padded rows: row groups G in
// {5, 6, 7, 8, 10}, offset planes K in {2, 3, 4, 5}, with and without the
// split evaluation, tracking words W in {1, 2}.
#include "binary_glynn.cuh"

namespace pg {

#define PG_BIN_SHAPES(X) \
    X(5, 2, 1) X(5, 2, 2) X(5, 3, 1) X(5, 3, 2) X(5, 4, 1) X(5, 4, 2) X(5, 5, 1) X(5, 5, 2) \
    X(6, 2, 1) X(6, 2, 2) X(6, 3, 1) X(6, 3, 2) X(6, 4, 1) X(6, 4, 2) X(6, 5, 1) X(6, 5, 2) \
    X(7, 2, 1) X(7, 2, 2) X(7, 3, 1) X(7, 3, 2) X(7, 4, 1) X(7, 4, 2) X(7, 5, 1) X(7, 5, 2) \
    X(8, 2, 1) X(8, 2, 2) X(8, 3, 1) X(8, 3, 2) X(8, 4, 1) X(8, 4, 2) X(8, 5, 1) X(8, 5, 2) \
    X(10, 2, 1) X(10, 2, 2) X(10, 3, 1) X(10, 3, 2) X(10, 4, 1) X(10, 4, 2) X(10, 5, 1) X(10, 5, 2) \

cudaError_t launch_binary_npad40(int G, int K, int W, const BinaryArgs &args, bool split,
                                  int blocks, cudaStream_t stream) {
#define PG_BIN_LAUNCH(GG, KK, WW) \
    if (G == GG && K == KK && W == WW) return launch_binary_glynn<40, GG, KK, WW>(args, split, blocks, stream);
    PG_BIN_SHAPES(PG_BIN_LAUNCH)
#undef PG_BIN_LAUNCH
    return cudaErrorInvalidValue;
}

int occupancy_binary_npad40(int G, int K, int W) {
#define PG_BIN_OCC(GG, KK, WW) \
    if (G == GG && K == KK && W == WW) return occupancy_binary_glynn<40, GG, KK, WW>();
    PG_BIN_SHAPES(PG_BIN_OCC)
#undef PG_BIN_OCC
    return 1;
}

}  // namespace pg
