// raster.cu -- per-tile rasterization of one frame (raster_common.cuh), one CTA per tile,
// instantiated for every supported tile shape.
#include "raster_common.cuh"

namespace sloth {

// One CTA per raster item (tile, slice); CTAs past the item count return at once.
template <int TW, int TH>
__global__ void __launch_bounds__(kRasterThreads, kRasterMinBlocks)
raster_kernel(FrameGeom g, FrameBuffers fb, BinBuffers bb, uint32_t ntiles, int depth_cull)
{
    __shared__ TileSmem<TW, TH> S;
    if (blockIdx.x >= bb.slice_offset[ntiles] || blockIdx.x >= bb.item_capacity) return;
    if (bb.tile_offset[ntiles] > bb.capacity) return;   // entries past the buffer: the host runs it again
    const uint2 it = bb.items[blockIdx.x];
    const uint32_t all = bb.tile_count[it.x];
    const uint32_t thr = bb.slice_offset[ntiles + 1], slice = bb.slice_offset[ntiles + 2];
    const bool split = all > thr;
    const uint32_t first = split ? it.y * slice : 0u;
    const uint32_t cnt = split ? min(slice, all - first) : all;
    raster_tile<TW, TH>(S, g, fb, (int)it.x, cnt, bb.entries + bb.tile_offset[it.x] + first, depth_cull, split);
}

cudaError_t launch_raster(const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                          int depth_cull, cudaStream_t s)
{
    const uint32_t ntiles = (uint32_t)(g.ntx * g.nty);
    if (ntiles == 0) return cudaSuccess;
    const uint32_t grid = bb.item_capacity;
#define SLOTH_RASTER_CASE(W_, H_)                                                              \
    if (g.tw == W_ && g.th == H_) {                                                            \
        raster_kernel<W_, H_><<<grid, kRasterThreads, 0, s>>>(g, fb, bb, ntiles, depth_cull);  \
        return cudaGetLastError();                                                             \
    }
    SLOTH_TILE_SHAPES(SLOTH_RASTER_CASE)
#undef SLOTH_RASTER_CASE
    return cudaErrorInvalidValue;
}

}  // namespace sloth
