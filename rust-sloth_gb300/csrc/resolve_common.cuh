// resolve_common.cuh -- per-cell resolve shared by the single-frame and batched kernels.
//
// For every frame cell c the reference's final value is the last of three kinds of
// write in draw order (src/rasterizer.rs:80-91):
//   - the last accepted depth write at cell c          (frame_buffer[id]   = pixel)
//   - the last accepted depth write at cell c-1         (frame_buffer[id+1] = pixel)
//   - in image mode, the newline sentinel of row y when c == y*w+1
// The last accepted depth write of a cell is its minimum key.  Draw order is compared
// as (triangle, sample row, sample column); a newline comes after every sample of its
// row.  The winner's depth, shade and char are recomputed from its record with the
// raster's exact operations, which also restores the sign of a -0.0 depth.
#pragma once

#include <climits>

#include "sloth_internal.cuh"
#include "sloth_kernels.h"

namespace sloth {

struct Cand {
    uint32_t tri;
    int32_t y, x;
    uint32_t cell;
};

__device__ __forceinline__ bool later(const Cand &a, const Cand &b)
{
    if (a.tri != b.tri) return a.tri > b.tri;
    if (a.y != b.y) return a.y > b.y;
    return a.x > b.x;
}

__device__ __forceinline__ uint64_t key_at(const FrameGeom &g, const FrameBuffers &fb, int r, int cc)
{
    const int tile = (r / g.th) * g.ntx + cc / g.tw;
    if (fb.tile_gen[tile] != fb.gen) return kEmptyKey;
    return fb.keys[(size_t)r * g.pitch + cc];
}

// Rebuild the winning write of depth cell (r, cc) from its key.
__device__ __forceinline__ Cand decode(const FrameGeom &g, const FrameBuffers &fb, uint64_t key,
                                       int r, int cc, float *z_out)
{
    Cand c;
    const uint32_t lo = (uint32_t)key;
    c.tri = lo >> 1;
    if (lo & 1u) {
        c.y = r;
        c.x = cc >> 1;
    } else {
        c.y = r - 1;
        c.x = (cc + g.w) >> 1;
    }
    const float4 *p = reinterpret_cast<const float4 *>(fb.records + c.tri);
    TriRecord rec;
    float4 *o = reinterpret_cast<float4 *>(&rec);
#pragma unroll
    for (int k = 0; k < 6; ++k) o[k] = __ldg(p + k);
    const EdgeVals e = eval_edges(rec, (float)c.x, (float)c.y);
    const float shade = fmul(rec.na, fadd(fadd(e.w0, e.w1), e.w2));
    if (z_out) *z_out = interp_z(rec.v1z, rec.dz2, rec.dz3, rec.a, e.w1, e.w2);
    c.cell = shade_char(shade) | (rec.rgb << 8);
    return c;
}

// Resolve frame cell c (and depth cell c when c < w*h) of one frame.
__device__ __forceinline__ void resolve_cell(const FrameGeom &g, const FrameBuffers &fb, uint64_t c)
{
    const uint64_t nz = (uint64_t)g.w * g.h;
    if (c >= nz) {
        fb.cells_out[c] = (uint32_t)' ';
        return;
    }
    const int r = (int)(c / g.w), cc = (int)(c - (uint64_t)r * g.w);
    bool have = false;
    Cand best{0, 0, 0, (uint32_t)' '};
    const uint64_t kc = key_at(g, fb, r, cc);
    if (kc != kEmptyKey) {
        float z;
        best = decode(g, fb, kc, r, cc, &z);
        have = true;
        fb.z_out[c] = z;
        fb.winner_out[c] = (int32_t)best.tri;
    } else {
        fb.z_out[c] = kFltMax;
        fb.winner_out[c] = -1;
    }
    if (c > 0) {
        const int pr = cc > 0 ? r : r - 1, pc = cc > 0 ? cc - 1 : g.w - 1;
        const uint64_t kp = key_at(g, fb, pr, pc);
        if (kp != kEmptyKey) {
            const Cand b = decode(g, fb, kp, pr, pc, nullptr);
            if (!have || later(b, best)) best = b;
            have = true;
        }
        if (g.image && (c - 1) % g.w == 0) {
            const uint64_t yn = (c - 1) / g.w;
            if (yn < (uint64_t)g.h) {
                const int32_t t = nltree_query(fb.nltree, g.nl_size, (int)yn);
                if (t >= 0) {
                    const Cand n{(uint32_t)t, (int32_t)yn, INT_MAX, (uint32_t)'\n'};
                    if (!have || later(n, best)) best = n;
                    have = true;
                }
            }
        }
    }
    fb.cells_out[c] = best.cell;
}

}  // namespace sloth
