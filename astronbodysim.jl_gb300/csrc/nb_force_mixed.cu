// nb_force_mixed.cu -- dispatch of the mixed-precision force and pack kernels
// (nb_force_mixed.cuh) by j-tile size.
#include "nb_force_mixed.cuh"

namespace nb {

extern template cudaError_t launch_force_mixed_tile<128>(int, bool, const Sources32&, const Targets&,
                                                         double, uint32_t*, int, int, int, cudaStream_t);
extern template cudaError_t launch_pack_tile<128>(const double*, const double*, const double*,
                                                  const double*, int64_t, const int32_t*, float4*,
                                                  TileOrigin*, float4*, cudaStream_t);
extern template cudaError_t launch_force_mixed_tile<256>(int, bool, const Sources32&, const Targets&,
                                                         double, uint32_t*, int, int, int, cudaStream_t);
extern template cudaError_t launch_pack_tile<256>(const double*, const double*, const double*,
                                                  const double*, int64_t, const int32_t*, float4*,
                                                  TileOrigin*, float4*, cudaStream_t);
extern template cudaError_t launch_force_mixed_tile<512>(int, bool, const Sources32&, const Targets&,
                                                         double, uint32_t*, int, int, int, cudaStream_t);
extern template cudaError_t launch_pack_tile<512>(const double*, const double*, const double*,
                                                  const double*, int64_t, const int32_t*, float4*,
                                                  TileOrigin*, float4*, cudaStream_t);

bool tile_size_ok(int tile_j) { return tile_j == 128 || tile_j == 256 || tile_j == 512; }

cudaError_t launch_pack(const double* x, const double* y, const double* z, const double* m,
                        int64_t n, const int32_t* perm, int tile_j, float4* pack,
                        TileOrigin* origin, float4* ext, cudaStream_t s) {
    switch (tile_j) {
        case 128: return launch_pack_tile<128>(x, y, z, m, n, perm, pack, origin, ext, s);
        case 256: return launch_pack_tile<256>(x, y, z, m, n, perm, pack, origin, ext, s);
        case 512: return launch_pack_tile<512>(x, y, z, m, n, perm, pack, origin, ext, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_force_mixed(int law, bool pot, const Sources32& src, const Targets& tg,
                               double G, uint32_t* err, int block, int ipt, cudaStream_t s,
                               int stages) {
    switch (src.tile_j) {
        case 128: return launch_force_mixed_tile<128>(law, pot, src, tg, G, err, block, ipt, stages, s);
        case 256: return launch_force_mixed_tile<256>(law, pot, src, tg, G, err, block, ipt, stages, s);
        case 512: return launch_force_mixed_tile<512>(law, pot, src, tg, G, err, block, ipt, stages, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace nb
