// record.cuh -- per-triangle setup shared by the single-frame and batched kernels.
//
// Restates, per triangle, src/rasterizer.rs:56-67 (aabb, sample range, a = 1/orient) and
// src/geometry.rs:37-56 (Triangle::aabb/normal) on already transformed vertices, with the
// reference's f32 operation order, then adds what the GPU path needs: the edge deltas,
// a proven-tight x bound, back-face culling and a depth lower bound.
#pragma once

#include "bounds.cuh"
#include "direct.cuh"
#include "sloth_internal.cuh"
#include "sloth_kernels.h"

namespace sloth {

// Smallest index in [lo,hi) where a monotone (false..true) predicate holds, hi if none.
template <class Pred>
__device__ __forceinline__ int first_true(int lo, int hi, Pred pred)
{
    while (lo < hi) {
        int mid = lo + ((hi - lo) >> 1);
        if (pred(mid)) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// True if no sample (px >= X, py in [y0,y1)) can be covered.  Along a row, an edge with
// dy > 0 is non-increasing in px and an edge with dy == 0 is constant, so if it is
// negative at X it stays negative for all px >= X.  At column X, each such edge is
// monotone in py (through C(py) = dx*(py-ay)), so the rows where it is negative form a
// prefix or a suffix of [y0,y1); the rows are all excluded iff those sets cover [y0,y1).
// Exact for records whose x,y are finite and below 1e18 (no overflow, no NaN).
__device__ __forceinline__ bool right_of_is_empty(const TriRecord &r, int X, int y0, int y1)
{
    const float px = (float)X;
    int prefix_end = y0;     // max end of negative prefixes
    int suffix_begin = y1;   // min begin of negative suffixes
    const float dxs[3] = {r.dx0, r.dx1, r.dx2};
    const float dys[3] = {r.dy0, r.dy1, r.dy2};
    const float axs[3] = {r.v2x, r.v3x, r.v1x};
    const float ays[3] = {r.v2y, r.v3y, r.v1y};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float dx = dxs[i], dy = dys[i], ax = axs[i], ay = ays[i];
        if (!(dy >= 0.0f)) continue;   // dy < 0: the edge grows with px, proves nothing
        auto neg = [&](int py) { return edge_eval(dx, dy, ax, ay, px, (float)py) < 0.0f; };
        if (dx > 0.0f) {
            // increasing in py: negative on a prefix
            int b = first_true(y0, y1, [&](int py) { return !neg(py); });
            prefix_end = max(prefix_end, b);
        } else if (dx < 0.0f) {
            // decreasing in py: negative on a suffix
            int s = first_true(y0, y1, [&](int py) { return neg(py); });
            suffix_begin = min(suffix_begin, s);
        } else {
            if (neg(y0)) return true;   // constant in py too
        }
    }
    return prefix_end >= suffix_begin;
}

__device__ __forceinline__ int sat_lo(float f, int cap)
{
    // Rust `f as usize` of ceil(max(v,1.0)) (>= 1, never NaN), clamped to cap.
    return f < (float)cap ? (int)f : cap;
}
__device__ __forceinline__ int sat_hi(float f)
{
    // Rust `f as usize` of ceil(min(v, dim-1)): NaN/negative -> 0, at most dim-1.
    return f > 0.0f ? (int)f : 0;
}

// Stores a record.  A triangle with no tile (culled, empty sample range) only ever has its
// sample range read -- by a context's overflow fold and the no-allocation raster, which
// stop there -- so only that row is written, with zeros in row 5 beside it (store_row4: a
// whole 32-byte sector, which the memory writes back without reading it first).  A direct
// triangle (direct.cuh) is never binned nor rasterized again: only the rows the resolve
// (0-1, 5) and a context's overflow fold (4) read are written.
__device__ __forceinline__ void store_record(TriRecord *dst, const TriRecord &r, uint32_t ntiles, bool direct = false)
{
    const int4 *src = reinterpret_cast<const int4 *>(&r);
    int4 *d = reinterpret_cast<int4 *>(dst);
    if (direct) {
        d[0] = src[0];
        d[1] = src[1];
        d[4] = src[4];
        d[5] = src[5];
    } else if (ntiles != 0) {
        *dst = r;
    } else {
        d[4] = make_int4(r.x0, r.xe, r.y0, r.y1);
        d[5] = make_int4(0, 0, 0, 0);
    }
}

// Record rows 4 (the sample range, row4) and 5 (zeros) of a triangle with nothing to
// rasterize (store_record).
__device__ __forceinline__ void store_row4(TriRecord *dst, int4 row4)
{
    int4 *d = reinterpret_cast<int4 *>(dst);
    d[4] = row4;
    d[5] = make_int4(0, 0, 0, 0);
}

// The first steps of build_record, for a setup kernel that sets triangles aside before the
// rest of their setup: the sample range and the back-face proof over the untightened range
// (the same operations as build_record).  Returns false for a triangle with an empty range
// or proven to cover no sample, with `row4` its record row 4 (x0, xe, y0, y1) -- all that
// is ever read of such a triangle; true when the triangle needs build_record.  Either way
// row4.z and row4.w are the rows [y0, y1) the record will hold.
__device__ __forceinline__ bool needs_setup(float4 p1, float4 p2, float4 p3, int w, int h, int4 &row4)
{
    TriRecord r;   // the fields orient_bound reads
    r.v1x = p1.x; r.v1y = p1.y; r.v2x = p2.x; r.v2y = p2.y; r.v3x = p3.x; r.v3y = p3.y;
    r.dx0 = fsub(p3.x, p2.x); r.dy0 = fsub(p3.y, p2.y);
    r.dx1 = fsub(p1.x, p3.x); r.dy1 = fsub(p1.y, p3.y);
    r.dx2 = fsub(p2.x, p1.x); r.dy2 = fsub(p2.y, p1.y);
    const float mnx = fminf(p1.x, fminf(p2.x, p3.x)), mny = fminf(p1.y, fminf(p2.y, p3.y));
    const float mxx = fmaxf(p1.x, fmaxf(p2.x, p3.x)), mxy = fmaxf(p1.y, fmaxf(p2.y, p3.y));
    r.x0 = sat_lo(ceilf(fmaxf(mnx, 1.0f)), w);
    r.y0 = sat_lo(ceilf(fmaxf(mny, 1.0f)), h);
    const int x1 = sat_hi(ceilf(fminf(fmul(mxx, 2.0f), (float)(w - 1))));
    r.y1 = sat_hi(ceilf(fminf(mxy, (float)(h - 1))));
    r.xe = x1;
    if (!(r.x0 < x1 && r.y0 < r.y1)) {
        row4 = make_int4(r.x0, x1, r.y0, r.y1);
        return false;
    }
    const float big = 1e18f;
    const bool finite = fabsf(p1.x) < big && fabsf(p1.y) < big && fabsf(p2.x) < big &&
                        fabsf(p2.y) < big && fabsf(p3.x) < big && fabsf(p3.y) < big;
    // the proof needs o < -err with err >= 0: a triangle whose computed orient o (the value
    // orient_bound computes first) is not negative is never proven empty, so the bound is
    // worked out only for the others (back faces, mostly)
    if (finite && edge_eval(r.dx2, r.dy2, r.v1x, r.v1y, r.v3x, r.v3y) < 0.0f && provably_empty(orient_bound(r))) {
        row4 = make_int4(r.x0, r.x0, r.y0, r.y1);
        return false;
    }
    row4 = make_int4(r.x0, x1, r.y0, r.y1);
    return true;
}

// A triangle's sample rows [y0, y1) packed for the newline kernels (FrameBuffers::rows):
// both lie in [0, h] and h is at most 65535.
__device__ __forceinline__ uint32_t pack_rows(int y0, int y1) { return (uint32_t)y0 | ((uint32_t)y1 << 16); }

// Face colour of triangle t: three bytes, packed as the record stores them.
__device__ __forceinline__ uint32_t load_rgb(const uint8_t *rgb, uint32_t t)
{
    const uint8_t *c = rgb + 3 * (size_t)t;
    return (uint32_t)__ldg(c) | ((uint32_t)__ldg(c + 1) << 8) | ((uint32_t)__ldg(c + 2) << 16);
}

// The queue between a setup block's two phases, in dynamic shared memory
// (setup_smem_bytes): per slot the triangle index, its packed colour and its three
// transformed vertices, as 11 arrays of cap words so that consecutive slots fall in
// different banks.  Phase 2 reads a queued triangle from here, not from global memory.
// setup_smem (direct.cuh) is indexed itself, which keeps the accesses 32-bit shared ones.

struct SetupStash {
    uint32_t cap;

    __device__ __forceinline__ void put(uint32_t s, uint32_t t, float4 p1, float4 p2, float4 p3, uint32_t c) const
    {
        setup_smem[s] = t;
        setup_smem[cap + s] = c;
        const float v[9] = {p1.x, p1.y, p1.z, p2.x, p2.y, p2.z, p3.x, p3.y, p3.z};
#pragma unroll
        for (int k = 0; k < 9; ++k) setup_smem[(2 + k) * cap + s] = __float_as_uint(v[k]);
    }
    __device__ __forceinline__ uint32_t get(uint32_t s, float4 &p1, float4 &p2, float4 &p3, uint32_t &c) const
    {
        float v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = __uint_as_float(setup_smem[(2 + k) * cap + s]);
        p1 = make_float4(v[0], v[1], v[2], 0.0f);
        p2 = make_float4(v[3], v[4], v[5], 0.0f);
        p3 = make_float4(v[6], v[7], v[8], 0.0f);
        c = setup_smem[cap + s];
        return setup_smem[s];
    }
};

// Queues triangle t when keep holds, with one shared atomic per warp (called by all 32
// lanes).  count is the block's running total of queued triangles and base its value when
// the chunk began, so the chunk's slots are 0, 1, ... in the stash.
__device__ __forceinline__ void stash_push(const SetupStash &st, uint32_t *count, uint32_t base, bool keep, uint32_t t,
                                           float4 p1, float4 p2, float4 p3, uint32_t c)
{
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    uint32_t first = 0;
    if (lane == 0) first = atomicAdd(count, (uint32_t)__popc(m));
    first = __shfl_sync(0xffffffffu, first, 0) - base;
    if (keep) st.put(first + __popc(m & ((1u << lane) - 1u)), t, p1, p2, p3, c);
}

// How the setup thread rasterizes a direct triangle (direct.cuh): its samples lie in rows
// [y0,y1) from column x0, up to column xend (exclusive); with exit_mask set, a row ends at
// the first column where an edge in the mask (bit i: edge i, those with dy > 0) is negative.
struct DirectWalk {
    bool direct;
    int xend;
    uint32_t exit_mask;
};

// The record of one triangle with transformed vertices p1, p2, p3 (xyz) and packed face
// colour rgb (load_rgb) in a w x h context, for a triangle needs_setup kept: a triangle
// with an empty range or proven to cover no sample over it (back faces) never gets here,
// so the back-face proof is not repeated.  With direct_max > 0, a triangle whose sample
// range holds at most direct_max samples is marked for the direct path (dw): such a
// triangle needs no proven tight bound nor depth bounds.  A finite triangle with an edge
// of dy > 0 is sized by its unproven right end floor(max.x)+1 (xe) and walked with early
// row exits up to the reference's bound; any other triangle is sized and walked by its
// stored range.  A triangle is direct exactly when is_direct(x0, xe, y0, y1, direct_max)
// holds for the stored range, so later kernels recognise it from row 4 alone.
__device__ __forceinline__ TriRecord build_record(float4 p1, float4 p2, float4 p3, uint32_t rgb, int w, int h,
                                                  int direct_max = 0, DirectWalk *dw = nullptr)
{
    TriRecord r;
    r.v1x = p1.x; r.v1y = p1.y; r.v2x = p2.x; r.v2y = p2.y; r.v3x = p3.x; r.v3y = p3.y;
    r.dx0 = fsub(p3.x, p2.x); r.dy0 = fsub(p3.y, p2.y);
    r.dx1 = fsub(p1.x, p3.x); r.dy1 = fsub(p1.y, p3.y);
    r.dx2 = fsub(p2.x, p1.x); r.dy2 = fsub(p2.y, p1.y);
    r.v1z = p1.z; r.dz2 = fsub(p2.z, p1.z); r.dz3 = fsub(p3.z, p1.z);
    // a = 1 / orient(v1, v2, v3)  (src/rasterizer.rs:67)
    const float orient = edge_eval(r.dx2, r.dy2, p1.x, p1.y, p3.x, p3.y);
    r.a = __fdiv_rn(1.0f, orient);
    // normal().z  (src/geometry.rs:49-56; norm of a 4-vector with w = 0)
    const float e1x = r.dx2, e1y = r.dy2, e1z = r.dz2;
    const float e2x = fsub(p3.x, p1.x), e2y = fsub(p3.y, p1.y), e2z = r.dz3;
    const float nx = fsub(fmul(e1y, e2z), fmul(e1z, e2y));
    const float ny = fsub(fmul(e1z, e2x), fmul(e1x, e2z));
    const float nz = fsub(fmul(e1x, e2y), fmul(e1y, e2x));
    const float norm2 = fadd(fadd(fmul(nx, nx), fmul(nz, nz)), fadd(fmul(ny, ny), fmul(0.0f, 0.0f)));
    const float n = __fsqrt_rn(fadd(0.0f, norm2));
    r.na = fmul(__fdiv_rn(nz, n), r.a);
    r.rgb = rgb;
    // aabb and sample range  (src/geometry.rs:37-42, src/rasterizer.rs:59-66)
    const float mnx = fminf(p1.x, fminf(p2.x, p3.x)), mny = fminf(p1.y, fminf(p2.y, p3.y));
    const float mxx = fmaxf(p1.x, fmaxf(p2.x, p3.x)), mxy = fmaxf(p1.y, fmaxf(p2.y, p3.y));
    r.x0 = sat_lo(ceilf(fmaxf(mnx, 1.0f)), w);
    r.y0 = sat_lo(ceilf(fmaxf(mny, 1.0f)), h);
    const int x1 = sat_hi(ceilf(fminf(fmul(mxx, 2.0f), (float)(w - 1))));
    r.y1 = sat_hi(ceilf(fminf(mxy, (float)(h - 1))));
    const float big = 1e18f;
    const bool finite = fabsf(p1.x) < big && fabsf(p1.y) < big && fabsf(p2.x) < big &&
                        fabsf(p2.y) < big && fabsf(p3.x) < big && fabsf(p3.y) < big;
    r.flags = finite ? kFlagFiniteXY : 0u;
    r.xe = x1;
    r.zlo = -INFINITY;
    if (dw) *dw = DirectWalk{false, 0, 0u};
    if (finite && r.x0 < x1 && r.y0 < r.y1) {
        if (direct_max > 0) {
            // Along a row an edge of dy > 0 is non-increasing in x (monotone correctly
            // rounded steps, finite values): once negative it stays negative, so a row walk
            // may stop there.  floor(max.x)+1 only sizes the triangle.
            const uint32_t mask = (r.dy0 > 0.0f ? 1u : 0u) | (r.dy1 > 0.0f ? 2u : 0u) | (r.dy2 > 0.0f ? 4u : 0u);
            const float xf = fadd(floorf(mxx), 1.0f);
            const int xa = xf <= (float)r.x0 ? r.x0 : (xf < (float)x1 ? (int)xf : x1);
            if (mask && is_direct(r.x0, xa, r.y0, r.y1, direct_max)) {
                r.xe = xa;
                if (dw) *dw = DirectWalk{true, x1, mask};
                return r;
            }
        }
        // first column strictly right of the triangle, not left of x0
        const float xf = fadd(floorf(mxx), 1.0f);
        if (xf < (float)x1) {
            const int X = xf <= (float)r.x0 ? r.x0 : (int)xf;
            if (right_of_is_empty(r, X, r.y0, r.y1)) {
                r.xe = X;
                r.flags |= kFlagTight;
            }
        }
        // cull triangles that provably cover no sample of the evaluated range (the range
        // right of xe is already proven empty, or xe is the reference's bound)
        if (r.x0 < r.xe) {
            const OrientBound ob = orient_bound(r);
            if (provably_empty(ob)) {
                r.xe = r.x0;
                r.flags |= kFlagCulled;
            } else {
                r.zlo = depth_lower_bound(r, ob);
            }
        }
    }
    // any other triangle with a range of at most direct_max samples is walked over it whole
    if (dw && direct_max > 0 && is_direct(r.x0, r.xe, r.y0, r.y1, direct_max)) *dw = DirectWalk{true, r.xe, 0u};
    return r;
}

// nalgebra Matrix4*Vector4 with w = 1: ((m0*x + m1*y) + m2*z) + m3*1, each step rounded.
__device__ __forceinline__ float row_dot(const float *m, float x, float y, float z)
{
    float acc = fmul(m[0], x);
    acc = fadd(fmul(m[1], y), acc);
    acc = fadd(fmul(m[2], z), acc);
    acc = fadd(fmul(m[3], 1.0f), acc);
    return acc;
}

// The triangle at position p of setup's order of the mesh (MeshDev::order).
__device__ __forceinline__ uint32_t mesh_triangle(const MeshDev &mesh, uint32_t p)
{
    return mesh.order ? __ldg(mesh.order + p) : p;
}

// The vertex indices of triangle t, at position p of setup's order.
__device__ __forceinline__ void mesh_corners(const MeshDev &mesh, uint32_t p, uint32_t t, uint32_t &i1, uint32_t &i2,
                                             uint32_t &i3)
{
    const uint32_t *ix = mesh.oidx ? mesh.oidx + 3 * (size_t)p : mesh.idx ? mesh.idx + 3 * (size_t)t : nullptr;
    if (ix) {
        i1 = __ldg(ix + 0);
        i2 = __ldg(ix + 1);
        i3 = __ldg(ix + 2);
    } else {
        i1 = 3 * t + 0; i2 = 3 * t + 1; i3 = 3 * t + 2;
    }
}

// One vertex transformed in place: (M*v).xyz with the vertex kernels' operations.
__device__ __forceinline__ float4 transform_vertex(const MeshDev &mesh, const Mat4 &M, uint32_t i)
{
    const float x = __ldg(mesh.x + i), y = __ldg(mesh.y + i), z = __ldg(mesh.z + i);
    return make_float4(row_dot(&M.m[0], x, y, z), row_dot(&M.m[4], x, y, z), row_dot(&M.m[8], x, y, z), 0.0f);
}

// Counts the small triangle's tiles (bin count pass) and returns the triangle's slot among
// the entries of its first tile.  A triangle's first tile (the first tile_hit in the loop
// order below, which fill_small_warp repeats) is counted in tile_count with one atomic per
// distinct tile of the warp, whose returned value gives each lane its slot; its other
// tiles are counted in tile_extra without a slot (the fill takes theirs from the tile's
// cursor).  Called by all 32 lanes (lanes with active false count nothing and get 0).
__device__ __forceinline__ uint32_t count_small_tiles_warp(bool active, const TriRecord &r, const Viewport &vp,
                                                           const TileSpan &sp, uint32_t *tile_count,
                                                           uint32_t *tile_extra)
{
    uint32_t first = 0xffffffffu;
    if (active) {
        auto hit = [&](int tr, int tc) {
            const uint32_t tile = tr * vp.ntx + tc;
            if (first == 0xffffffffu) first = tile;
            else atomicAdd(&tile_extra[tile], 1u);
        };
        for (int tr = sp.TU.ya; tr < sp.TU.yb; ++tr)
            for (int tc = sp.TU.xa; tc < sp.TU.xb; ++tc)
                if (tile_hit(r, vp, sp.U, sp.W, tr, tc)) hit(tr, tc);
        for (int tr = sp.TW.ya; tr < sp.TW.yb; ++tr)
            for (int tc = sp.TW.xa; tc < sp.TW.xb; ++tc) {
                if (in_rect(sp.TU, tr, tc)) continue;
                if (tile_hit(r, vp, sp.U, sp.W, tr, tc)) hit(tr, tc);
            }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, first);
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (first != 0xffffffffu && lane == leader) base = atomicAdd(&tile_count[first], (uint32_t)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    return first != 0xffffffffu ? base + (uint32_t)__popc(peers & ((1u << lane) - 1u)) : 0u;
}

}  // namespace sloth
