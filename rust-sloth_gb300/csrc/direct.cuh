// direct.cuh -- rasterizing a small triangle straight into the frame's global depth keys.
//
// Most triangles of a finely tessellated mesh cover a handful of samples.  Binning them
// (a tile count, a scan, an entry per tile, a sort in the tile's CTA) costs far more than
// their samples do.  A triangle whose sample range [x0,xe) x [y0,y1) holds at most
// FrameGeom::direct_max samples is therefore rasterized by the warp that set it up: the
// warp runs the reference's loop body (src/rasterizer.rs:69-86) over the range and folds
// each covered sample's depth key into the global key of its target cell with a 64-bit
// atomicMin.  The minimum of a cell's keys does not depend on the order of the folds, so
// the result is the same as folding the triangle in its tile's CTA; the tile raster later
// loads those keys and folds the binned triangles on top.
//
// The global keys of every tile must be valid for the current generation (cleared to the
// empty key) before the first direct fold of a frame.
#pragma once

#include <climits>

#include "sloth_internal.cuh"

namespace sloth {

// True when a triangle with sample range [x0,xe) x [y0,y1) is rasterized directly.
__host__ __device__ __forceinline__ bool is_direct(int x0, int xe, int y0, int y1, int direct_max)
{
    return x0 < xe && y0 < y1 && (uint32_t)(xe - x0) * (uint32_t)(y1 - y0) <= (uint32_t)direct_max;
}

// The direct triangles of a warp folded together (called by all 32 lanes; lanes with
// mine false bring none).  A triangle's samples lie in rows [y0, y1) from column x0 up to
// xend (exclusive); with exit_mask set a row ends at the first column where an edge of the
// mask (bit i: edge i, edges whose value only falls along a row) is negative.  Sample
// (x, y) writes depth cell y*w + 2x (src/rasterizer.rs:80): row y, column 2x when 2x < w,
// else row y+1, column 2x-w, stored at key_col of its column for tile width tw.  Each
// triangle's walked samples are its rows times the columns [x0, xs): xs = xend for a
// triangle walked over its stored range (exit_mask 0); with row exits, xs =
// min(r.xe + 1, xend), the unproven end plus one probe column.  The warp walks
// the concatenation of all its triangles' samples 32 at a time, each lane finding its
// triangle by a binary search over the running ends, so that the lanes stay busy and one
// reduction instruction covers neighbouring samples of a few triangles (fewer memory
// requests).  A covered sample is never past a row's exit (an exit edge, once negative,
// stays negative along the row), so walking every column up to the probe folds the same
// samples as a row walk with exits.  When the probe column still has no exit edge
// negative, the lane that tested it walks the rest of that row, up to its first exit.
// The warp stages its triangles in kDirectStageWords words of the setup kernels' dynamic
// shared memory from word `stage` on (structure of arrays: field f of lane l at f*32 + l,
// so lanes reading one triangle share a broadcast and different triangles fall in
// different banks).
constexpr int kDirectFields = 23;
constexpr int kDirectStageWords = kDirectFields * 32;

// The setup kernels' dynamic shared memory (record.cuh: SetupStash; then one direct stage
// per warp).  Indexing the array itself keeps the accesses 32-bit shared ones.
extern __shared__ uint32_t setup_smem[];

__device__ __forceinline__ uint32_t direct_raster_warp(bool mine, const TriRecord &r, uint32_t gtri, int w, int pitch,
                                                      int tw, unsigned long long *keys, int xend, uint32_t exit_mask,
                                                      uint32_t stage)
{
    const int lane = threadIdx.x & 31;
    float *sf = reinterpret_cast<float *>(setup_smem + stage);
    int *si = reinterpret_cast<int *>(setup_smem + stage);
    int n = 0;
    if (mine) {
        const bool probe = exit_mask != 0u && r.xe < xend;   // r.xe <= xend always
        const int xs = probe ? r.xe + 1 : xend;
        const int cols = xs - r.x0;
        n = cols * (r.y1 - r.y0);
        const float v[16] = {r.v1x, r.v1y, r.v2x, r.v2y, r.v3x, r.v3y, r.dx0, r.dy0,
                             r.dx1, r.dy1, r.dx2, r.dy2, r.v1z, r.dz2, r.dz3, r.a};
#pragma unroll
        for (int f = 0; f < 16; ++f) sf[f * 32 + lane] = v[f];
        si[16 * 32 + lane] = r.x0;
        si[17 * 32 + lane] = r.y0;
        si[18 * 32 + lane] = cols;
        si[19 * 32 + lane] = probe ? r.xe : INT_MAX;
        si[20 * 32 + lane] = xend;
        si[21 * 32 + lane] = (int)exit_mask;
        si[22 * 32 + lane] = (int)gtri;
    }
    int end = n;   // running end of the samples up to this lane's triangle
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, end, d);
        if (lane >= d) end += o;
    }
    const int total = __shfl_sync(0xffffffffu, end, 31), first = end - n;
    __syncwarp();
    uint32_t frags = 0;
    for (int base = 0; base < total; base += 32) {
        const int k = base + lane;
        // the triangle of sample k: the number of lanes whose samples end at or before k
        int src = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
            if (__shfl_sync(0xffffffffu, end, src + step - 1) <= k) src += step;
        const int i = k - __shfl_sync(0xffffffffu, first, src);
        if (k >= total) continue;
        const int cols = si[18 * 32 + src];
        // i / cols from a reciprocal: i + 0.5 is at least 0.5 from a multiple of cols, far
        // beyond the rounding error for the sizes a direct triangle has
        const int row = (int)(((float)i + 0.5f) * __frcp_rn((float)cols));
        const int x = si[16 * 32 + src] + (i - row * cols), y = si[17 * 32 + src] + row;
        TriRecord t;
        t.v1x = sf[0 * 32 + src]; t.v1y = sf[1 * 32 + src]; t.v2x = sf[2 * 32 + src]; t.v2y = sf[3 * 32 + src];
        t.v3x = sf[4 * 32 + src]; t.v3y = sf[5 * 32 + src];
        t.dx0 = sf[6 * 32 + src]; t.dy0 = sf[7 * 32 + src]; t.dx1 = sf[8 * 32 + src]; t.dy1 = sf[9 * 32 + src];
        t.dx2 = sf[10 * 32 + src]; t.dy2 = sf[11 * 32 + src];
        t.v1z = sf[12 * 32 + src]; t.dz2 = sf[13 * 32 + src]; t.dz3 = sf[14 * 32 + src]; t.a = sf[15 * 32 + src];
        const uint32_t id = (uint32_t)si[22 * 32 + src];
        unsigned long long *rowu = keys + (size_t)y * pitch, *rown = rowu + pitch;
        auto fold = [&](int xx, const EdgeVals &e) {
            if (e.w0 >= 0.0f && e.w1 >= 0.0f && e.w2 >= 0.0f) {
                ++frags;
                const float z = interp_z(t.v1z, t.dz2, t.dz3, t.a, e.w1, e.w2);
                if (z < kFltMax) {
                    const uint32_t nw = 2 * xx < w ? 1u : 0u;
                    red_min_u64((nw ? rowu : rown) + key_col(nw ? 2 * xx : 2 * xx - w, tw),
                                (unsigned long long)make_key(z, id, nw));
                }
            }
        };
        const EdgeVals e = eval_edges(t, (float)x, (float)y);
        fold(x, e);
        if (x == si[19 * 32 + src]) {
            const uint32_t mask = (uint32_t)si[21 * 32 + src];
            const uint32_t neg = (e.w0 < 0.0f ? 1u : 0u) | (e.w1 < 0.0f ? 2u : 0u) | (e.w2 < 0.0f ? 4u : 0u);
            if (!(neg & mask)) {
                // the row goes on past the probe column (rare: edge values that round to
                // >= 0 right of max.x): walk it up to its first exit
                const EdgeRows c = edge_rows(t, (float)y);
                const int xe2 = si[20 * 32 + src];
                for (int xx = x + 1; xx < xe2; ++xx) {
                    const EdgeVals e2 = eval_edges_row(t, c, (float)xx);
                    const uint32_t n2 = (e2.w0 < 0.0f ? 1u : 0u) | (e2.w1 < 0.0f ? 2u : 0u) | (e2.w2 < 0.0f ? 4u : 0u);
                    if (n2 & mask) break;
                    fold(xx, e2);
                }
            }
        }
    }
    __syncwarp();   // the stage is reused by the warp's next call
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
