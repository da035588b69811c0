// Instantiations of binary_glynn_kernel with 32 padded rows (G in
// {5, 6, 7, 8, 10}, bit planes B in {3, 4, 5, 6}).
#include "binary_glynn.cuh"

namespace pg {

#define PG_BIN_SHAPES(X) \
    X(5, 3) X(5, 4) X(5, 5) X(5, 6) X(6, 3) X(6, 4) X(6, 5) X(6, 6) \
    X(7, 3) X(7, 4) X(7, 5) X(7, 6) X(8, 3) X(8, 4) X(8, 5) X(8, 6) \
    X(10, 3) X(10, 4) X(10, 5) X(10, 6)

cudaError_t launch_binary_npad32(int G, int B, const BinaryArgs &args, int blocks,
                                  cudaStream_t stream) {
#define PG_BIN_LAUNCH(GG, BB) \
    if (G == GG && B == BB) return launch_binary_glynn<32, GG, BB>(args, blocks, stream);
    PG_BIN_SHAPES(PG_BIN_LAUNCH)
#undef PG_BIN_LAUNCH
    return cudaErrorInvalidValue;
}

int occupancy_binary_npad32(int G, int B) {
#define PG_BIN_OCC(GG, BB) \
    if (G == GG && B == BB) return occupancy_binary_glynn<32, GG, BB>();
    PG_BIN_SHAPES(PG_BIN_OCC)
#undef PG_BIN_OCC
    return 1;
}

cudaError_t launch_binary_npad40(int G, int B, const BinaryArgs &args, int blocks,
                                  cudaStream_t stream);
cudaError_t launch_binary_npad48(int G, int B, const BinaryArgs &args, int blocks,
                                  cudaStream_t stream);
int occupancy_binary_npad40(int G, int B);
int occupancy_binary_npad48(int G, int B);

int binary_npad(int n) { return n <= 32 ? 32 : n <= 40 ? 40 : n <= 48 ? 48 : 0; }

bool binary_compiled(int NPAD, int G, int B) {
    const bool g = G == 5 || G == 6 || G == 7 || G == 8 || G == 10;
    return (NPAD == 32 || NPAD == 40 || NPAD == 48) && g && B >= 3 && B <= 6;
}

cudaError_t launch_binary_any(int NPAD, int G, int B, const BinaryArgs &args, int blocks,
                              cudaStream_t stream) {
    if (!binary_compiled(NPAD, G, B)) return cudaErrorInvalidValue;
    return NPAD == 32 ? launch_binary_npad32(G, B, args, blocks, stream)
         : NPAD == 40 ? launch_binary_npad40(G, B, args, blocks, stream)
                      : launch_binary_npad48(G, B, args, blocks, stream);
}

int occupancy_binary_any(int NPAD, int G, int B) {
    return NPAD == 32 ? occupancy_binary_npad32(G, B)
         : NPAD == 40 ? occupancy_binary_npad40(G, B)
                      : occupancy_binary_npad48(G, B);
}

}  // namespace pg
