// sloth_internal.cuh -- device-side definitions shared by the GB300 kernels.
//
// Exactness: every float operation on the path goes through the IEEE round-to-nearest
// intrinsics (__fadd_rn, __fsub_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn), which the
// compiler never contracts into FMAs.  The translation units are also built with
// -fmad=false and without -ftz, so subnormals behave as in the reference.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sloth {

// ---------------------------------------------------------------------------------
// Exact f32 arithmetic (Rust semantics: no contraction, round to nearest even).
// ---------------------------------------------------------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// Block barrier.  __syncthreads compiles to an aligned barrier, which expects every warp
// to arrive converged; after lane-dependent code (single-lane sections, loops whose trip
// count differs between lanes) a warp is first reconverged with __syncwarp.  Without it a
// warp can be counted before all its lanes arrive, and the barriers of the block fall out
// of step.
__device__ __forceinline__ void block_sync()
{
    __syncwarp();
    __syncthreads();
}

constexpr float kFltMax = 3.40282347e+38f;
constexpr uint64_t kEmptyKey = ~0ull;
constexpr uint32_t kSmallMaxTilesDev = 16;   // triangles over more tiles are binned by warps

// orient(a, b, p) of src/rasterizer.rs:30-32 with the edge constants precomputed:
// (bx-ax)*(py-ay) - (by-ay)*(px-ax) where dx = bx-ax, dy = by-ay.
__device__ __forceinline__ float edge_eval(float dx, float dy, float ax, float ay, float px,
                                          float py)
{
    return fsub(fmul(dx, fsub(py, ay)), fmul(dy, fsub(px, ax)));
}

// default_shader, src/rasterizer.rs:5-27.
__device__ __forceinline__ uint32_t shade_char(float s)
{
    if (s <= 0.20f) return '.';
    if (s <= 0.30f) return ':';
    if (s <= 0.40f) return '-';
    if (s <= 0.50f) return '=';
    if (s <= 0.60f) return '+';
    if (s <= 0.70f) return '*';
    if (s <= 0.80f) return '#';
    if (s <= 0.90f) return '%';
    if (s <= 1.0f) return '@';
    return ' ';
}

// ---------------------------------------------------------------------------------
// Triangle record written by the setup kernel, one per triangle drawn since clear,
// indexed by the global draw index.  96 bytes = 6 x 16-byte rows.
//   edge 0: a = v2, b = v3   (w0 = orient(v2, v3, p))
//   edge 1: a = v3, b = v1   (w1 = orient(v3, v1, p))
//   edge 2: a = v1, b = v2   (w2 = orient(v1, v2, p))
// Rows 0-1 (one 32-byte sector) hold all the resolve reads of a winning triangle in the
// common case: the vertices' x and y (the edge deltas are their differences), the shade
// factor and the colour.
// ---------------------------------------------------------------------------------
struct __align__(16) TriRecord {
    float v1x, v1y, v2x, v2y;       // row 0
    float v3x, v3y;                 // row 1
    float na;                       //        normal().z * a (shade = na * ((w0+w1)+w2))
    uint32_t rgb;                   //        r | g<<8 | b<<16
    float dx0, dy0, dx1, dy1;       // row 2: dx0 = v3x - v2x, dx1 = v1x - v3x, dx2 = v2x - v1x
    float dx2, dy2;                 // row 3
    uint32_t flags;                 //        kFlag*
    float zlo;                      //        lower bound of every depth the raster can compute
                                    //        for this triangle, or -inf (bounds.cuh)
    int32_t x0, xe, y0, y1;         // row 4: sample rect [x0,xe) x [y0,y1) (xe: tight or loose)
    float v1z, dz2, dz3, a;         // row 5: z = v1z + a*((w1*dz2) + (w2*dz3))
};
static_assert(sizeof(TriRecord) == 96, "record layout");

// The whole record in one round trip (six 16-byte loads).
__device__ __forceinline__ TriRecord load_record(const TriRecord *__restrict__ recs, uint32_t i)
{
    const float4 *p = reinterpret_cast<const float4 *>(recs + i);
    TriRecord r;
    float4 *o = reinterpret_cast<float4 *>(&r);
#pragma unroll
    for (int k = 0; k < 6; ++k) o[k] = __ldg(p + k);
    return r;
}

constexpr uint32_t kFlagFiniteXY = 1u;   // |x|,|y| of all vertices < 1e18: edge functions are
                                         // monotone and overflow-free, corner tests are exact
constexpr uint32_t kFlagTight = 2u;      // xe was tightened below the reference's x bound
constexpr uint32_t kFlagCulled = 4u;     // proven to cover no sample (xe = x0)

// Sample-space edge values for one record at integer sample (px, py).
struct EdgeVals {
    float w0, w1, w2;
};
__device__ __forceinline__ EdgeVals eval_edges(const TriRecord &r, float px, float py)
{
    EdgeVals e;
    e.w0 = edge_eval(r.dx0, r.dy0, r.v2x, r.v2y, px, py);
    e.w1 = edge_eval(r.dx1, r.dy1, r.v3x, r.v3y, px, py);
    e.w2 = edge_eval(r.dx2, r.dy2, r.v1x, r.v1y, px, py);
    return e;
}

// The same three edge values with each edge's row term fl(dx*fl(py-ay)) computed once per
// row: edge_eval(dx, dy, ax, ay, px, py) == fsub(row, fmul(dy, fsub(px, ax))) exactly (the
// same operations, the same order).
struct EdgeRows {
    float c0, c1, c2;
};
__device__ __forceinline__ EdgeRows edge_rows(const TriRecord &r, float py)
{
    return EdgeRows{fmul(r.dx0, fsub(py, r.v2y)), fmul(r.dx1, fsub(py, r.v3y)), fmul(r.dx2, fsub(py, r.v1y))};
}
__device__ __forceinline__ EdgeVals eval_edges_row(const TriRecord &r, const EdgeRows &c, float px)
{
    EdgeVals e;
    e.w0 = fsub(c.c0, fmul(r.dy0, fsub(px, r.v2x)));
    e.w1 = fsub(c.c1, fmul(r.dy1, fsub(px, r.v3x)));
    e.w2 = fsub(c.c2, fmul(r.dy2, fsub(px, r.v1x)));
    return e;
}

// 64-bit minimum into global memory without a returned value (a fire-and-forget
// reduction: the thread does not wait for it).
__device__ __forceinline__ void red_min_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("red.global.min.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// z of src/rasterizer.rs:77-79.
__device__ __forceinline__ float interp_z(float v1z, float dz2, float dz3, float a, float w1,
                                          float w2)
{
    return fadd(v1z, fmul(a, fadd(fmul(w1, dz2), fmul(w2, dz3))));
}

// Depth key: ordered(canonical z) in the high word, (draw index << 1 | !wrapped) in the
// low word.  atomicMin over keys selects the reference's last successful writer: the
// smallest z, and among equal z (-0 == +0) the earliest in draw order (triangle, then
// row; the wrapped sample of a cell comes from the row above, so it is earlier).
__device__ __forceinline__ uint32_t ordered_z(float z)
{
    uint32_t b = __float_as_uint(z);
    if (b == 0x80000000u) b = 0u;                     // -0 -> +0
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
// The float of an ordered depth (ordered_z's inverse, -0 read as +0).
__device__ __forceinline__ float float_of_ordered(uint32_t o)
{
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
__device__ __forceinline__ uint64_t make_key(float z, uint32_t tri, uint32_t not_wrapped)
{
    return ((uint64_t)ordered_z(z) << 32) | (uint64_t)((tri << 1) | not_wrapped);
}

// ---------------------------------------------------------------------------------
// Target-cell tiling.  Sample (x,y) writes depth cell id = y*w + 2x (src/rasterizer.rs:80):
// row y, column 2x when 2x < w ("unwrapped"), else row y+1, column 2x-w ("wrapped").
// Tiles partition depth cells; every writer of a cell lands in the cell's tile.
//
// Key layout.  Within every aligned run of tw cells of a row (a tile row) the keys of the
// even columns come first, then those of the odd columns: column c is stored at key_col(c).
// Unwrapped samples write even columns, wrapped ones columns of w's parity, so when w is
// even only the first half of each tile row is ever written (its other half is neither
// copied, cleared nor read), and a warp's samples along a row hit consecutive keys.
// ---------------------------------------------------------------------------------
__host__ __device__ __forceinline__ int key_col(int c, int tw)
{
    return (c & ~(tw - 1)) | ((c & 1) ? (tw >> 1) : 0) | ((c & (tw - 1)) >> 1);
}
// Keys of one tile row that are ever written: half of them when w is even.
__host__ __device__ __forceinline__ int live_keys_per_row(int w, int tw) { return (w & 1) ? tw : tw >> 1; }

struct Viewport {
    int32_t w, h;           // sample grid / depth cells
    int32_t image;
    int32_t tw, th;         // tile size in cells (tw even)
    int32_t ntx, nty;       // tile grid
    int32_t pitch;          // key-buffer row pitch in cells (= ntx*tw)
};

struct Rect {
    int32_t xa, xb, ya, yb;   // [xa,xb) x [ya,yb)
    __device__ __forceinline__ bool empty() const { return xa >= xb || ya >= yb; }
};

// Unwrapped / wrapped sample sub-rectangles of a record's sample rect.
__device__ __forceinline__ Rect unwrapped_part(const Viewport &vp, int x0, int xe, int y0, int y1)
{
    int xw = (vp.w + 1) >> 1;
    return Rect{x0, min(xe, xw), y0, y1};
}
__device__ __forceinline__ Rect wrapped_part(const Viewport &vp, int x0, int xe, int y0, int y1)
{
    int xw = (vp.w + 1) >> 1;
    return Rect{max(x0, xw), xe, y0, y1};
}

// Tile-index rectangle [txa,txb) x [tya,tyb) covered by a sample part.
__device__ __forceinline__ Rect tiles_of_unwrapped(const Viewport &vp, const Rect &s)
{
    return Rect{(2 * s.xa) / vp.tw, (2 * (s.xb - 1)) / vp.tw + 1, s.ya / vp.th,
                (s.yb - 1) / vp.th + 1};
}
__device__ __forceinline__ Rect tiles_of_wrapped(const Viewport &vp, const Rect &s)
{
    return Rect{(2 * s.xa - vp.w) / vp.tw, (2 * (s.xb - 1) - vp.w) / vp.tw + 1,
                (s.ya + 1) / vp.th, s.yb / vp.th + 1};
}

// Samples of tile (tr, tc) that fall in a record part.
__device__ __forceinline__ Rect clip_unwrapped(const Viewport &vp, const Rect &s, int tr, int tc)
{
    int c0 = tc * vp.tw, r0 = tr * vp.th;
    Rect r;
    r.xa = max(s.xa, c0 >> 1);
    r.xb = min(s.xb, (c0 + vp.tw) >> 1);
    r.ya = max(s.ya, r0);
    r.yb = min(s.yb, r0 + vp.th);
    return r;
}
__device__ __forceinline__ Rect clip_wrapped(const Viewport &vp, const Rect &s, int tr, int tc)
{
    int c0 = tc * vp.tw, r0 = tr * vp.th;
    Rect r;
    r.xa = max(s.xa, (c0 + vp.w + 1) >> 1);          // 2x - w >= c0
    r.xb = min(s.xb, (c0 + vp.tw + vp.w + 1) >> 1);  // 2x - w <  c0 + tw
    r.ya = max(s.ya, r0 - 1);
    r.yb = min(s.yb, r0 + vp.th - 1);
    return r;
}

// Exact rejection: the maximum of one edge function over a sample rectangle is reached
// at one corner, because w = fl(C(py) - U(px)) with C monotone in py and U monotone in
// px (each a chain of correctly rounded monotone operations).  If that maximum is
// negative for any edge, no sample of the rectangle is covered.  Valid only for
// records with kFlagFiniteXY.
__device__ __forceinline__ bool rect_may_cover(const TriRecord &r, const Rect &s)
{
    float xl = (float)s.xa, xr = (float)(s.xb - 1), yl = (float)s.ya, yh = (float)(s.yb - 1);
    float w0 = edge_eval(r.dx0, r.dy0, r.v2x, r.v2y, r.dy0 > 0.0f ? xl : xr, r.dx0 > 0.0f ? yh : yl);
    float w1 = edge_eval(r.dx1, r.dy1, r.v3x, r.v3y, r.dy1 > 0.0f ? xl : xr, r.dx1 > 0.0f ? yh : yl);
    float w2 = edge_eval(r.dx2, r.dy2, r.v1x, r.v1y, r.dy2 > 0.0f ? xl : xr, r.dx2 > 0.0f ? yh : yl);
    return !(w0 < 0.0f || w1 < 0.0f || w2 < 0.0f);
}

__device__ __forceinline__ uint32_t tile_hit(const TriRecord &r, const Viewport &vp, const Rect &U,
                                             const Rect &W, int tr, int tc)
{
    const bool exact = (r.flags & kFlagFiniteXY) != 0;
    if (!U.empty()) {
        Rect c = clip_unwrapped(vp, U, tr, tc);
        if (!c.empty() && (!exact || rect_may_cover(r, c))) return 1;
    }
    if (!W.empty()) {
        Rect c = clip_wrapped(vp, W, tr, tc);
        if (!c.empty() && (!exact || rect_may_cover(r, c))) return 1;
    }
    return 0;
}


// Sample parts and tile rectangles of a record, and its binning class.
struct TileSpan {
    Rect U, W;          // unwrapped / wrapped sample parts (may be empty)
    Rect TU, TW;        // their tile rectangles (empty when the part is)
    uint32_t ntiles;    // tiles of both rectangles (an upper bound of the tiles hit)
    bool large;         // binned by a warp instead of a thread
};
__device__ __forceinline__ TileSpan tile_span_of(const Viewport &vp, int x0, int xe, int y0, int y1)
{
    TileSpan sp;
    sp.U = sp.W = sp.TU = sp.TW = Rect{0, 0, 0, 0};
    sp.ntiles = 0;
    if (x0 < xe && y0 < y1) {
        sp.U = unwrapped_part(vp, x0, xe, y0, y1);
        sp.W = wrapped_part(vp, x0, xe, y0, y1);
        if (!sp.U.empty()) {
            sp.TU = tiles_of_unwrapped(vp, sp.U);
            sp.ntiles += (sp.TU.xb - sp.TU.xa) * (sp.TU.yb - sp.TU.ya);
        } else {
            sp.U = Rect{0, 0, 0, 0};
        }
        if (!sp.W.empty()) {
            sp.TW = tiles_of_wrapped(vp, sp.W);
            sp.ntiles += (sp.TW.xb - sp.TW.xa) * (sp.TW.yb - sp.TW.ya);
        } else {
            sp.W = Rect{0, 0, 0, 0};
        }
    }
    sp.large = sp.ntiles > kSmallMaxTilesDev;
    return sp;
}
__device__ __forceinline__ TileSpan tile_span(const Viewport &vp, const TriRecord &r)
{
    return tile_span_of(vp, r.x0, r.xe, r.y0, r.y1);
}

__device__ __forceinline__ bool in_rect(const Rect &t, int tr, int tc)
{
    return tr >= t.ya && tr < t.yb && tc >= t.xa && tc < t.xb;
}

// Newline segment tree over n (power of two) rows: fold draw index v into the rows
// [y0,y1) with the canonical O(log n) node decomposition.  `always` forces the atomic
// (shared-memory trees); otherwise a read filters updates that cannot raise a node.
__device__ __forceinline__ void nltree_update(int32_t *tree, int n, int y0, int y1, int32_t v, bool always)
{
    int l = y0 + n, r = y1 + n;
    while (l < r) {
        if (l & 1) {
            if (always || *(volatile int32_t *)&tree[l] < v) atomicMax(&tree[l], v);
            ++l;
        }
        if (r & 1) {
            --r;
            if (always || *(volatile int32_t *)&tree[r] < v) atomicMax(&tree[r], v);
        }
        l >>= 1;
        r >>= 1;
    }
}

// The last newline writer of row y: the maximum over the leaf-to-root path (-1: none).
__device__ __forceinline__ int32_t nltree_query(const int32_t *tree, int n, int y)
{
    int32_t t = -1;
    for (uint32_t i = (uint32_t)y + (uint32_t)n; i >= 1; i >>= 1) t = max(t, tree[i]);
    return t;
}

}  // namespace sloth
