// bin_common.cuh -- per-triangle binning steps shared by the single-frame and batched
// kernels.  A triangle is listed in every target-cell tile whose cells it can write
// (tile_hit: an exact corner test cannot rule the tile out).  The order inside a tile
// list does not matter: the raster's 64-bit atomicMin recovers the draw order.
#pragma once

#include "bounds.cuh"
#include "sloth_internal.cuh"

namespace sloth {

// A tile entry: the ordered depth lower bound in the high word (the raster sorts on it,
// front to back), the draw index in bits 0..30 and, in bit 31, whether the triangle has
// wrapped samples in this tile (they write other cells than unwrapped samples).
__device__ __forceinline__ uint64_t entry_key(float zlo, uint32_t gtri, bool wrapped)
{
    return ((uint64_t)ordered_z(zlo) << 32) | gtri | (wrapped ? 0x80000000u : 0u);
}

// Triangles over more than kSmallMaxTilesDev tiles are binned by warps.  Those over more
// than kBigTiles tiles ("big") are split among kBigParts warps (part p takes every
// kBigParts-th group of 32 tiles), so that no lane walks hundreds of tiles in a row; the
// others take one warp each.  Big triangles are queued from the front of the queue and
// the others from the back, and the warp items list every big part first, so that the
// longest work starts first.
constexpr uint32_t kBigTiles = 256;
constexpr uint32_t kBigParts = 16;

// Queue slot of a large triangle of this warp (called by all 32 lanes; -1 for lanes
// without one): one atomic per class and warp.
__device__ __forceinline__ int large_slot(bool large, uint32_t ntiles, uint32_t *large_count, uint32_t cap)
{
    const int lane = threadIdx.x & 31;
    const bool big = large && ntiles > kBigTiles;
    const unsigned mb = __ballot_sync(0xffffffffu, big), mm = __ballot_sync(0xffffffffu, large && !big);
    uint32_t b0 = 0, m0 = 0;
    if (lane == 0) {
        if (mb) b0 = atomicAdd(&large_count[0], (uint32_t)__popc(mb));
        if (mm) m0 = atomicAdd(&large_count[1], (uint32_t)__popc(mm));
    }
    b0 = __shfl_sync(0xffffffffu, b0, 0);
    m0 = __shfl_sync(0xffffffffu, m0, 0);
    const unsigned lt = (1u << lane) - 1u;
    if (big) return (int)(b0 + __popc(mb & lt));
    if (large) return (int)(cap - 1u - (m0 + __popc(mm & lt)));
    return -1;
}

// Warp item i of the large queue: its queue slot, part and part count; false past the end.
__device__ __forceinline__ bool large_item(uint32_t i, const uint32_t *large_count, uint32_t cap, uint32_t &q,
                                           uint32_t &part, uint32_t &nparts)
{
    const uint32_t nb = large_count[0] * kBigParts;
    if (i < nb) {
        q = i / kBigParts;
        part = i % kBigParts;
        nparts = kBigParts;
        return true;
    }
    if (i - nb >= large_count[1]) return false;
    q = cap - 1u - (i - nb);
    part = 0;
    nparts = 1;
    return true;
}

__device__ __forceinline__ uint32_t large_items(const uint32_t *large_count)
{
    return large_count[0] * kBigParts + large_count[1];
}

// One warp walks part `part` of `nparts` of a large triangle's tile rectangles: counts (kFill
// false, in tile_cursor: entries whose slots come from the cursor after the scan) or writes
// its entries (kFill true), with a per-tile depth bound (tighter than the triangle-wide one).
// The sample range (16 bytes) decides first whether the part has tiles at all; only then
// is the whole record read.
template <bool kFill>
__device__ __forceinline__ void bin_large_warp(const TriRecord *rec, uint32_t gtri, const Viewport &vp,
                                               uint32_t *tile_count, uint32_t *tile_cursor,
                                               uint64_t *entries, uint32_t capacity, int lane, uint32_t part,
                                               uint32_t nparts)
{
    const int4 xr = __ldg(reinterpret_cast<const int4 *>(rec) + 4);
    const TileSpan sp = tile_span_of(vp, xr.x, xr.y, xr.z, xr.w);
    const int nu = (sp.TU.xb - sp.TU.xa) * (sp.TU.yb - sp.TU.ya);
    const int nw = (sp.TW.xb - sp.TW.xa) * (sp.TW.yb - sp.TW.ya);
    const int uw = sp.TU.xb - sp.TU.xa, ww = sp.TW.xb - sp.TW.xa;
    if ((int)part * 32 >= nu + nw) return;
    const TriRecord r = *rec;
    const OrientBound ob = orient_bound(r);
    for (int k = (int)part * 32 + lane; k < nu + nw; k += 32 * (int)nparts) {
        int tr, tc;
        if (k < nu) {
            tr = sp.TU.ya + k / uw;
            tc = sp.TU.xa + k % uw;
        } else {
            tr = sp.TW.ya + (k - nu) / ww;
            tc = sp.TW.xa + (k - nu) % ww;
            if (in_rect(sp.TU, tr, tc)) continue;
        }
        if (!tile_hit(r, vp, sp.U, sp.W, tr, tc)) continue;
        const uint32_t tile = tr * vp.ntx + tc;
        if (kFill) {
            float zlo = r.zlo;
            const Rect cu = sp.U.empty() ? Rect{0, 0, 0, 0} : clip_unwrapped(vp, sp.U, tr, tc);
            const Rect cw = sp.W.empty() ? Rect{0, 0, 0, 0} : clip_wrapped(vp, sp.W, tr, tc);
            if (r.flags & kFlagFiniteXY) {
                float zt = INFINITY;
                if (!cu.empty()) zt = fminf(zt, rect_depth_lower_bound(r, ob, cu));
                if (!cw.empty()) zt = fminf(zt, rect_depth_lower_bound(r, ob, cw));
                zlo = fmaxf(zlo, zt);
            }
            const uint32_t slot = atomicAdd(&tile_cursor[tile], 1u);
            if (slot < capacity) entries[slot] = entry_key(zlo, gtri, !cw.empty());
        } else {
            // counted among the tile's entries without a slot: the cursor array holds those
            // counts until the scan (count_small_tiles_warp)
            atomicAdd(&tile_cursor[tile], 1u);
        }
    }
}

// Writes a small triangle's entries: the one in its first tile at the slot the count pass
// gave it (slot1, after the tile's first tile_offset), the others at slots taken from the
// tiles' cursors.  A lane's tiles are tile_base + the frame-local index (the lanes of one
// warp may belong to different frames).
__device__ __forceinline__ void fill_small_warp(bool active, const TriRecord &r, uint32_t gtri, const Viewport &vp,
                                                const TileSpan &sp, const uint32_t *tile_offset,
                                                uint32_t *tile_cursor, uint64_t *entries, uint32_t capacity,
                                                uint32_t slot1, uint32_t tile_base = 0)
{
    if (!active) return;
    bool first = true;
    auto put = [&](int tr, int tc) {
        const bool wrapped = !sp.W.empty() && !clip_wrapped(vp, sp.W, tr, tc).empty();
        const uint32_t tile = tile_base + tr * vp.ntx + tc;
        uint32_t slot;
        if (first) {
            slot = tile_offset[tile] + slot1;
            first = false;
        } else {
            slot = atomicAdd(&tile_cursor[tile], 1u);
        }
        if (slot < capacity) entries[slot] = entry_key(r.zlo, gtri, wrapped);
    };
    for (int tr = sp.TU.ya; tr < sp.TU.yb; ++tr)
        for (int tc = sp.TU.xa; tc < sp.TU.xb; ++tc)
            if (tile_hit(r, vp, sp.U, sp.W, tr, tc)) put(tr, tc);
    for (int tr = sp.TW.ya; tr < sp.TW.yb; ++tr)
        for (int tc = sp.TW.xa; tc < sp.TW.xb; ++tc) {
            if (in_rect(sp.TU, tr, tc)) continue;
            if (tile_hit(r, vp, sp.U, sp.W, tr, tc)) put(tr, tc);
        }
}

}  // namespace sloth
