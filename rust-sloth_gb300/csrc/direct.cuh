// direct.cuh -- rasterizing a small triangle straight into the frame's global depth keys.
//
// Most triangles of a finely tessellated mesh cover a handful of samples.  Binning them
// (a tile count, a scan, an entry per tile, a sort in the tile's CTA) costs far more than
// their samples do.  A triangle whose sample range [x0,xe) x [y0,y1) holds at most
// FrameGeom::direct_max samples is therefore rasterized by the thread that set it up: it
// runs the reference's loop body (src/rasterizer.rs:69-86) over its range and folds each
// covered sample's depth key into the global key of its target cell with a 64-bit
// atomicMin.  The minimum of a cell's keys does not depend on the order of the folds, so
// the result is the same as folding the triangle in its tile's CTA; the tile raster later
// loads those keys and folds the binned triangles on top.
//
// The global keys of every tile must be valid for the current generation (cleared to the
// empty key) before the first direct fold of a frame.
#pragma once

#include "sloth_internal.cuh"

namespace sloth {

// True when a triangle with sample range [x0,xe) x [y0,y1) is rasterized directly.
__host__ __device__ __forceinline__ bool is_direct(int x0, int xe, int y0, int y1, int direct_max)
{
    return x0 < xe && y0 < y1 && (uint32_t)(xe - x0) * (uint32_t)(y1 - y0) <= (uint32_t)direct_max;
}

// The samples of rows [y0,y1) from column x0 to xend (exclusive) in the reference's
// row-major order (the order does not matter for the result); a row ends early at the
// first column where an edge of exit_mask (bit i: edge i) is negative -- edges whose value
// only falls along the row, so no later sample of the row can be covered.  Sample (x, y)
// writes depth cell y*w + 2x (src/rasterizer.rs:80): row y, column 2x when 2x < w, else
// row y+1, column 2x-w, stored at key_col of its column for tile width tw.  Returns the
// covered samples.
__device__ __forceinline__ uint32_t direct_raster(const TriRecord &r, uint32_t gtri, int w, int pitch, int tw,
                                                 unsigned long long *keys, int xend, uint32_t exit_mask)
{
    uint32_t frags = 0;
    for (int y = r.y0; y < r.y1; ++y) {
        const EdgeRows c = edge_rows(r, (float)y);
        unsigned long long *rowu = keys + (size_t)y * pitch, *rown = rowu + pitch;
        for (int x = r.x0; x < xend; ++x) {
            const EdgeVals e = eval_edges_row(r, c, (float)x);
            const uint32_t neg = (e.w0 < 0.0f ? 1u : 0u) | (e.w1 < 0.0f ? 2u : 0u) | (e.w2 < 0.0f ? 4u : 0u);
            if (neg & exit_mask) break;
            if (e.w0 >= 0.0f && e.w1 >= 0.0f && e.w2 >= 0.0f) {
                ++frags;
                const float z = interp_z(r.v1z, r.dz2, r.dz3, r.a, e.w1, e.w2);
                if (z < kFltMax) {
                    // unwrapped: row y, column 2x; wrapped: row y+1, column 2x-w
                    const uint32_t nw = 2 * x < w ? 1u : 0u;
                    red_min_u64((nw ? rowu : rown) + key_col(nw ? 2 * x : 2 * x - w, tw),
                                (unsigned long long)make_key(z, gtri, nw));
                }
            }
        }
    }
    return frags;
}

// Adds the warp's covered-sample counts to the frame's counter with one atomic (all 32
// lanes call it).
__device__ __forceinline__ void add_frags_warp(uint32_t frags, unsigned long long *counter)
{
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) frags += __shfl_xor_sync(0xffffffffu, frags, d);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(counter, (unsigned long long)frags);
}

}  // namespace sloth
