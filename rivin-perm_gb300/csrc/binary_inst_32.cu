// Instantiations of binary_glynn_kernel with 32 padded rows: row groups G in
// {5, 6, 7, 8, 10}, offset planes K in {2, 3, 4, 5}, with and without the
// split evaluation, tracking words W in {1}.
#include "binary_glynn.cuh"

namespace pg {

#define PG_BIN_SHAPES(X) \
    X(5, 2, 1) X(5, 3, 1) X(5, 4, 1) X(5, 5, 1) \
    X(6, 2, 1) X(6, 3, 1) X(6, 4, 1) X(6, 5, 1) \
    X(7, 2, 1) X(7, 3, 1) X(7, 4, 1) X(7, 5, 1) \
    X(8, 2, 1) X(8, 3, 1) X(8, 4, 1) X(8, 5, 1) \
    X(10, 2, 1) X(10, 3, 1) X(10, 4, 1) X(10, 5, 1) \

cudaError_t launch_binary_npad32(int G, int K, int W, const BinaryArgs &args, bool split,
                                  int blocks, cudaStream_t stream) {
#define PG_BIN_LAUNCH(GG, KK, WW) \
    if (G == GG && K == KK && W == WW) return launch_binary_glynn<32, GG, KK, WW>(args, split, blocks, stream);
    PG_BIN_SHAPES(PG_BIN_LAUNCH)
#undef PG_BIN_LAUNCH
    return cudaErrorInvalidValue;
}

int occupancy_binary_npad32(int G, int K, int W) {
#define PG_BIN_OCC(GG, KK, WW) \
    if (G == GG && K == KK && W == WW) return occupancy_binary_glynn<32, GG, KK, WW>();
    PG_BIN_SHAPES(PG_BIN_OCC)
#undef PG_BIN_OCC
    return 1;
}

cudaError_t launch_binary_npad40(int G, int K, int W, const BinaryArgs &args, bool split,
                                  int blocks, cudaStream_t stream);
cudaError_t launch_binary_npad48(int G, int K, int W, const BinaryArgs &args, bool split,
                                  int blocks, cudaStream_t stream);
int occupancy_binary_npad40(int G, int K, int W);
int occupancy_binary_npad48(int G, int K, int W);

int binary_npad(int n) { return n <= 32 ? 32 : n <= 40 ? 40 : n <= 48 ? 48 : 0; }

bool binary_compiled(int NPAD, int G, int K, int W) {
    const bool g = G == 5 || G == 6 || G == 7 || G == 8 || G == 10;
    const bool w = W == 1 || (W == 2 && NPAD > 32);
    return (NPAD == 32 || NPAD == 40 || NPAD == 48) && g && K >= 2 && K <= 5 && w;
}

cudaError_t launch_binary_any(int NPAD, int G, int K, int W, const BinaryArgs &args, bool split,
                              int blocks, cudaStream_t stream) {
    if (!binary_compiled(NPAD, G, K, W)) return cudaErrorInvalidValue;
    return NPAD == 32 ? launch_binary_npad32(G, K, W, args, split, blocks, stream)
         : NPAD == 40 ? launch_binary_npad40(G, K, W, args, split, blocks, stream)
                      : launch_binary_npad48(G, K, W, args, split, blocks, stream);
}

int occupancy_binary_any(int NPAD, int G, int K, int W) {
    return NPAD == 32 ? occupancy_binary_npad32(G, K, W)
         : NPAD == 40 ? occupancy_binary_npad40(G, K, W)
                      : occupancy_binary_npad48(G, K, W);
}

}  // namespace pg
