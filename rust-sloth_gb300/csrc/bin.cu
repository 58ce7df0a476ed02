// bin.cu -- binning of one frame's triangles into target-cell tiles.
//
// The reference visits every sample of every triangle's range in one sequential loop
// (src/rasterizer.rs:69-70).  Here each triangle is listed in the tiles whose depth
// cells it can write: count (setup kernel for small triangles, one warp per large
// triangle here), exclusive scan over tiles, then fill (bin_common.cuh).
#include "bin_common.cuh"
#include "sloth_kernels.h"

namespace sloth {

__device__ __forceinline__ Viewport vp_of(const FrameGeom &g)
{
    return Viewport{g.w, g.h, g.image, g.tw, g.th, g.ntx, g.nty, g.pitch};
}

// One warp per queued large triangle.
template <bool kFill>
__global__ void __launch_bounds__(256)
bin_large_kernel(uint32_t tri_base, FrameGeom g, FrameBuffers fb, BinBuffers bb)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nq = *bb.large_count;
    const Viewport vp = vp_of(g);
    for (uint32_t q = warp; q < nq; q += nwarps) {
        const uint32_t gtri = tri_base + bb.large_queue[q];
        bin_large_warp<kFill>(fb.records[gtri], gtri, vp, bb.tile_count, bb.tile_cursor, bb.entries,
                              bb.capacity, lane);
    }
}

// Exclusive scan of tile counts by one block; offsets[n] = total; cursors = offsets.
__global__ void __launch_bounds__(1024) bin_scan_kernel(uint32_t n, BinBuffers bb)
{
    __shared__ uint32_t warp_sums[32];
    const uint32_t tid = threadIdx.x;
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t lo = min(n, tid * per), hi = min(n, lo + per);
    uint32_t local = 0;
    for (uint32_t i = lo; i < hi; ++i) local += bb.tile_count[i];
    // inclusive scan of `local` across the block
    const int lane = tid & 31, wid = tid >> 5;
    uint32_t v = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += o;
    }
    if (lane == 31) warp_sums[wid] = v;
    block_sync();
    if (wid == 0) {
        uint32_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t o = __shfl_up_sync(0xffffffffu, s, d);
            if (lane >= d) s += o;
        }
        warp_sums[lane] = s;
    }
    block_sync();
    uint32_t run = v - local + (wid > 0 ? warp_sums[wid - 1] : 0u);   // exclusive prefix
    for (uint32_t i = lo; i < hi; ++i) {
        bb.tile_offset[i] = run;
        bb.tile_cursor[i] = run;
        run += bb.tile_count[i];
    }
    if (tid == blockDim.x - 1) bb.tile_offset[n] = warp_sums[(blockDim.x >> 5) - 1];
}

// One thread per triangle of the draw: small triangles write their tile entries.
__global__ void __launch_bounds__(256)
bin_fill_kernel(uint32_t ntri, uint32_t tri_base, FrameGeom g, FrameBuffers fb, BinBuffers bb)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const uint32_t gtri = tri_base + t;
    const TriRecord r = fb.records[gtri];
    const Viewport vp = vp_of(g);
    const TileSpan sp = tile_span(vp, r);
    if (sp.large || sp.ntiles == 0) return;
    fill_small(r, gtri, vp, sp, bb.tile_cursor, bb.entries, bb.capacity);
}

static int large_grid()
{
    return 2 * 152;   // two CTAs of 8 warps per SM; the warps stride over the queue
}

cudaError_t launch_bin_count_large(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                                   const BinBuffers &bb, cudaStream_t s)
{
    bin_large_kernel<false><<<large_grid(), 256, 0, s>>>(tri_base, g, fb, bb);
    return cudaGetLastError();
}

cudaError_t launch_bin_scan(uint32_t ntiles, const BinBuffers &bb, cudaStream_t s)
{
    bin_scan_kernel<<<1, 1024, 0, s>>>(ntiles, bb);
    return cudaGetLastError();
}

cudaError_t launch_bin_fill(uint32_t ntri, uint32_t tri_base, const FrameGeom &g,
                            const FrameBuffers &fb, const BinBuffers &bb, cudaStream_t s)
{
    if (ntri == 0) return cudaSuccess;
    bin_fill_kernel<<<(ntri + 255) / 256, 256, 0, s>>>(ntri, tri_base, g, fb, bb);
    return cudaGetLastError();
}

cudaError_t launch_bin_fill_large(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                                  const BinBuffers &bb, cudaStream_t s)
{
    bin_large_kernel<true><<<large_grid(), 256, 0, s>>>(tri_base, g, fb, bb);
    return cudaGetLastError();
}

}  // namespace sloth
