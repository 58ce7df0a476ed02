// raster.cu -- per-tile rasterization of one frame (raster_common.cuh), one CTA per tile,
// instantiated for every supported tile shape.
#include "raster_common.cuh"

namespace sloth {

template <int TW, int TH>
__global__ void __launch_bounds__(kRasterThreads)
raster_kernel(FrameGeom g, FrameBuffers fb, BinBuffers bb, int depth_cull)
{
    __shared__ TileSmem<TW, TH> S;
    const int tile = blockIdx.x;
    const uint32_t cnt = bb.tile_count[tile];
    if (cnt == 0) return;
    raster_tile<TW, TH>(S, g, fb, tile, cnt, bb.entries + bb.tile_offset[tile], depth_cull);
}

cudaError_t launch_raster(const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                          int depth_cull, cudaStream_t s)
{
    const int ntiles = g.ntx * g.nty;
    if (ntiles == 0) return cudaSuccess;
#define SLOTH_RASTER_CASE(W_, H_)                                                              \
    if (g.tw == W_ && g.th == H_) {                                                            \
        raster_kernel<W_, H_><<<ntiles, kRasterThreads, 0, s>>>(g, fb, bb, depth_cull);        \
        return cudaGetLastError();                                                             \
    }
    SLOTH_TILE_SHAPES(SLOTH_RASTER_CASE)
#undef SLOTH_RASTER_CASE
    return cudaErrorInvalidValue;
}

}  // namespace sloth
