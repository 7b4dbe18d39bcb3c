// nb_force_mixed_t256.cu -- the mixed-precision force kernels with j-tiles of
// 256 sources (one translation unit per tile size, compiled in parallel).
#include "nb_force_mixed.cuh"

namespace nb {

template cudaError_t launch_force_mixed_tile<256>(int, bool, const Sources32&, const Targets&, double,
                                                 uint32_t*, int, int, int, cudaStream_t);
template cudaError_t launch_pack_tile<256>(const double*, const double*, const double*,
                                          const double*, int64_t, const int32_t*, float4*,
                                          TileOrigin*, float4*, cudaStream_t);

}  // namespace nb
