// raster.cu -- per-tile rasterization of one frame (raster_common.cuh), one CTA per tile,
// instantiated for every supported tile shape.
#include "direct.cuh"
#include "raster_common.cuh"

namespace sloth {

// One CTA per raster item (tile, slice); CTAs past the item count return at once.
template <int TW, int TH>
__global__ void __launch_bounds__(kRasterThreads, kRasterMinBlocks)
raster_kernel(FrameGeom g, FrameBuffers fb, BinBuffers bb, uint32_t ntiles, int depth_cull)
{
    __shared__ TileSmem<TW, TH> S;
    if (blockIdx.x >= bb.slice_offset[ntiles] || blockIdx.x >= bb.item_capacity) return;
    if (bb.tile_offset[ntiles] > bb.capacity) return;   // entries past the buffer: launch_overflow does it
    const uint2 it = bb.items[blockIdx.x];
    const uint32_t all = bb.tile_count[it.x];
    const uint32_t thr = bb.slice_offset[ntiles + 1], slice = bb.slice_offset[ntiles + 2];
    const bool split = all > thr;
    const uint32_t first = split ? it.y * slice : 0u;
    const uint32_t cnt = split ? min(slice, all - first) : all;
    raster_barrier_init(S);
    uint32_t phase = 0;
    raster_tile<TW, TH>(S, g, fb, (int)it.x, cnt, bb.entries + bb.tile_offset[it.x] + first, depth_cull, phase,
                        split);
}

// Overflow fallback, step 1: grid-stride over tiles, one warp per tile; a tile whose keys
// belong to an older generation gets empty keys and the current generation.
__global__ void __launch_bounds__(256) overflow_tiles_kernel(FrameGeom g, FrameBuffers fb, BinBuffers bb,
                                                             uint32_t ntiles)
{
    if (bb.tile_offset[ntiles] <= bb.capacity) return;
    const int lane = threadIdx.x & 31;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles; t += nwarps) {
        if (fb.tile_gen[t] == fb.gen) continue;
        const int tr = (int)t / g.ntx, tc = (int)t - tr * g.ntx;
        unsigned long long *k0 = reinterpret_cast<unsigned long long *>(fb.keys) + (size_t)tr * g.th * g.pitch +
                                 (size_t)tc * g.tw;
        for (int i = lane; i < g.th * g.tw; i += 32) {
            const int r = i / g.tw, c = i - r * g.tw;
            k0[(size_t)r * g.pitch + c] = kEmptyKey;
        }
        __syncwarp();
        if (lane == 0) fb.tile_gen[t] = fb.gen;
    }
}

// Overflow fallback, step 2: one warp per triangle of the draw (grid-stride); a triangle
// the tiles would have rasterized (not culled, not direct) has every sample of its range
// tested, the lanes striding over the range, and its covered samples' keys folded into the
// global keys with a 64-bit atomicMin (the same minimum as the tile raster's).
__global__ void __launch_bounds__(256) overflow_raster_kernel(uint32_t ntri, uint32_t tri_base, FrameGeom g,
                                                              FrameBuffers fb, BinBuffers bb, uint32_t ntiles)
{
    if (bb.tile_offset[ntiles] <= bb.capacity) return;
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
                    atomicMin(keys + (size_t)row * g.pitch + col, (unsigned long long)make_key(z, gtri, nw));
                }
            }
        }
    }
    add_frags_warp(frags, fb.fragments);
}

cudaError_t launch_overflow(uint32_t ntri, uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                            const BinBuffers &bb, cudaStream_t s)
{
    const uint32_t ntiles = (uint32_t)(g.ntx * g.nty);
    if (ntiles == 0 || ntri == 0) return cudaSuccess;
    const int grid = 2 * device_sm_count();
    overflow_tiles_kernel<<<grid, 256, 0, s>>>(g, fb, bb, ntiles);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    overflow_raster_kernel<<<4 * grid, 256, 0, s>>>(ntri, tri_base, g, fb, bb, ntiles);
    return cudaGetLastError();
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
