// raster.cu -- per-tile rasterization of one frame (raster_common.cuh), one CTA per tile,
// instantiated for every supported tile shape.
#include "direct.cuh"
#include "raster_common.cuh"

namespace sloth {

// Overflow fallback of a draw whose tile entries outgrew the entry buffer (its fill wrote
// what fitted): one warp per triangle of the draw (grid-stride over the raster grid's
// warps); a triangle the tiles would have rasterized (not culled, not direct) has every
// sample of its range tested, the lanes striding over the range, and its covered samples'
// keys folded into the global keys with a 64-bit atomicMin -- the same minimum as the tile
// raster's.  bin_items_kernel has made every tile's keys current before.
__device__ __forceinline__ void overflow_fold(uint32_t ntri, uint32_t tri_base, const FrameGeom &g,
                                              const FrameBuffers &fb)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(fb.keys);
    uint32_t frags = 0;
    for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntri; t += nwarps) {
        const uint32_t gtri = tri_base + t;
        const int4 xr = __ldg(reinterpret_cast<const int4 *>(fb.records + gtri) + 4);
        if (!(xr.x < xr.y && xr.z < xr.w) || is_direct(xr.x, xr.y, xr.z, xr.w, g.direct_max)) continue;
        const TriRecord r = load_record(fb.records, gtri);
        const uint32_t bw = (uint32_t)(r.xe - r.x0);
        const uint64_t area = (uint64_t)bw * (uint32_t)(r.y1 - r.y0);
        for (uint64_t k = lane; k < area; k += 32) {
            const int y = r.y0 + (int)(k / bw), x = r.x0 + (int)(k % bw);
            const EdgeVals e = eval_edges(r, (float)x, (float)y);
            if (e.w0 >= 0.0f && e.w1 >= 0.0f && e.w2 >= 0.0f) {
                ++frags;
                const float z = interp_z(r.v1z, r.dz2, r.dz3, r.a, e.w1, e.w2);
                if (z < kFltMax) {
                    const uint32_t nw = 2 * x < g.w ? 1u : 0u;
                    const int row = nw ? y : y + 1, col = nw ? 2 * x : 2 * x - g.w;
                    red_min_u64(keys + (size_t)row * g.pitch + key_col(col, g.tw),
                                (unsigned long long)make_key(z, gtri, nw));
                }
            }
        }
    }
    add_frags_warp(frags, fb.fragments);
}

// One CTA per raster item (tile, slice); CTAs past the item count return at once.  When the
// draw's entries outgrew the buffer, every CTA of the grid takes part in overflow_fold
// instead.
template <int TW, int TH>
__global__ void __launch_bounds__(kRasterThreads, kRasterMinBlocks)
raster_kernel(FrameGeom g, FrameBuffers fb, BinBuffers bb, uint32_t ntiles, int depth_cull, uint32_t ntri,
              uint32_t tri_base)
{
    __shared__ TileSmem<TW, TH> S;
    if (bb.tile_offset[ntiles] > bb.capacity) {
        overflow_fold(ntri, tri_base, g, fb);
        return;
    }
    if (blockIdx.x >= bb.slice_offset[ntiles] || blockIdx.x >= bb.item_capacity) return;
    const uint2 it = bb.items[blockIdx.x];
    const uint32_t all = bb.tile_count[it.x];
    const uint32_t thr = bb.slice_offset[ntiles + 1], slice = bb.slice_offset[ntiles + 2];
    const bool split = all > thr;
    const uint32_t first = split ? it.y * slice : 0u;
    const uint32_t cnt = split ? min(slice, all - first) : all;
    uint32_t phase = 0;
    raster_tile<TW, TH>(S, g, fb, (int)it.x, cnt, bb.entries + bb.tile_offset[it.x] + first, depth_cull, phase,
                        split);
}

cudaError_t launch_raster(const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                          int depth_cull, uint32_t ntri, uint32_t tri_base, cudaStream_t s)
{
    const uint32_t ntiles = (uint32_t)(g.ntx * g.nty);
    if (ntiles == 0) return cudaSuccess;
    const uint32_t grid = bb.item_capacity;
#define SLOTH_RASTER_CASE(W_, H_)                                                              \
    if (g.tw == W_ && g.th == H_) {                                                            \
        raster_kernel<W_, H_><<<grid, kRasterThreads, 0, s>>>(g, fb, bb, ntiles, depth_cull, ntri, tri_base); \
        return cudaGetLastError();                                                             \
    }
    SLOTH_TILE_SHAPES(SLOTH_RASTER_CASE)
#undef SLOTH_RASTER_CASE
    return cudaErrorInvalidValue;
}

}  // namespace sloth
