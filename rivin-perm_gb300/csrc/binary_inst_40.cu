// Instantiations of binary_glynn_kernel with 40 padded rows (G in
// {5, 6, 7, 8, 10}, bit planes B in {3, 4, 5, 6}).
#include "binary_glynn.cuh"

namespace pg {

#define PG_BIN_SHAPES(X) \
    X(5, 3) X(5, 4) X(5, 5) X(5, 6) X(6, 3) X(6, 4) X(6, 5) X(6, 6) \
    X(7, 3) X(7, 4) X(7, 5) X(7, 6) X(8, 3) X(8, 4) X(8, 5) X(8, 6) \
    X(10, 3) X(10, 4) X(10, 5) X(10, 6)

cudaError_t launch_binary_npad40(int G, int B, const BinaryArgs &args, int blocks,
                                  cudaStream_t stream) {
#define PG_BIN_LAUNCH(GG, BB) \
    if (G == GG && B == BB) return launch_binary_glynn<40, GG, BB>(args, blocks, stream);
    PG_BIN_SHAPES(PG_BIN_LAUNCH)
#undef PG_BIN_LAUNCH
    return cudaErrorInvalidValue;
}

int occupancy_binary_npad40(int G, int B) {
#define PG_BIN_OCC(GG, BB) \
    if (G == GG && B == BB) return occupancy_binary_glynn<40, GG, BB>();
    PG_BIN_SHAPES(PG_BIN_OCC)
#undef PG_BIN_OCC
    return 1;
}

}  // namespace pg
