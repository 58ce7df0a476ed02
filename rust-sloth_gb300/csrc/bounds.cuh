// bounds.cuh -- rigorous floating-point bounds used to skip work without changing results.
//
// Every skip decision on the raster path (a culled triangle, a rejected tile, a triangle
// hidden behind a tile's current depths) is taken only when a bound proves that the
// reference's computation, done exactly as the raster does it, could not have written
// anything.  The bounds use directed rounding (__f*_ru / __f*_rd) so that every
// intermediate is itself a bound, and generous error factors (8u where the classical
// orient2d analysis needs 3u + 16u^2, u = 2^-24).
#pragma once

#include "sloth_internal.cuh"

namespace sloth {

constexpr float kU8 = 4.76837158e-07f;    // 8u
constexpr float kU4 = 2.38418579e-07f;    // 4u
constexpr float kTiny = 1e-37f;           // absolute slack for underflow

// Upper bound of |fl(q - a)| over integers q in [qa, qb].
__device__ __forceinline__ float ub_absdiff(float a, int qa, int qb)
{
    const float fa = (float)qa, fb = (float)qb;
    const float m = fmaxf(fmaxf(__fsub_ru(fa, a), __fsub_ru(a, fa)), fmaxf(__fsub_ru(fb, a), __fsub_ru(a, fb)));
    return __fmul_ru(fmaxf(m, 0.0f), 1.0f + 1.1920929e-07f);
}

// Error bound of a computed 2x2 determinant fl(fl(p*fl(d1)) - fl(q*fl(d2))) given upper
// bounds of its two product magnitudes.
__device__ __forceinline__ float det_err_ru(float absL, float absR)
{
    return __fadd_ru(__fmul_ru(kU8, __fadd_ru(absL, absR)), kTiny);
}

// Error bounds b_i of the three computed edge functions over the record's evaluation
// rectangle [x0,xe) x [y0,y1): |w_i(p) - E_i(p)| <= b_i with E_i the exact value.
struct EdgeBounds {
    float b[3];
    float sum;
};
__device__ __forceinline__ EdgeBounds edge_error_bounds(const TriRecord &r)
{
    const float dxs[3] = {r.dx0, r.dx1, r.dx2};
    const float dys[3] = {r.dy0, r.dy1, r.dy2};
    const float axs[3] = {r.v2x, r.v3x, r.v1x};
    const float ays[3] = {r.v2y, r.v3y, r.v1y};
    EdgeBounds eb;
    eb.sum = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float py = ub_absdiff(ays[i], r.y0, r.y1 - 1);
        const float px = ub_absdiff(axs[i], r.x0, r.xe - 1);
        eb.b[i] = det_err_ru(__fmul_ru(fabsf(dxs[i]), py), __fmul_ru(fabsf(dys[i]), px));
        eb.sum = __fadd_ru(eb.sum, eb.b[i]);
    }
    return eb;
}

// The computed orient(v1,v2,v3) of src/rasterizer.rs:67 and the error bound of it plus
// the edge bounds: err >= b_o + b0 + b1 + b2.
struct OrientBound {
    float o, err;
    EdgeBounds eb;
};
__device__ __forceinline__ OrientBound orient_bound(const TriRecord &r)
{
    OrientBound ob;
    ob.o = edge_eval(r.dx2, r.dy2, r.v1x, r.v1y, r.v3x, r.v3y);
    const float absL = fabsf(fmul(r.dx2, fsub(r.v3y, r.v1y)));
    const float absR = fabsf(fmul(r.dy2, fsub(r.v3x, r.v1x)));
    ob.eb = edge_error_bounds(r);
    ob.err = __fadd_ru(det_err_ru(absL, absR), ob.eb.sum);
    return ob;
}

// True if no sample of the evaluation rectangle can have all three computed edge
// functions >= 0.  For any point p the exact edge functions satisfy E0+E1+E2 = O (the
// exact orient).  w_i >= 0 implies E_i >= -b_i, so coverage needs O >= -(b0+b1+b2), and
// O <= o + b_o.  Hence o < -err proves the triangle covers nothing (back faces, mostly).
__device__ __forceinline__ bool provably_empty(const OrientBound &ob) { return ob.o < -ob.err; }

__device__ __forceinline__ bool depth_bound_usable(const TriRecord &r, const OrientBound &ob)
{
    return ob.o > 0.0f && fabsf(r.v1z) < 1e30f && fabsf(r.dz2) < 1e30f && fabsf(r.dz3) < 1e30f &&
           r.a > 0.0f && r.a < INFINITY && __fdiv_ru(ob.err, ob.o) < 1e6f;
}

// Lower bound of every depth the raster can compute for a covered sample of the triangle
// (src/rasterizer.rs:77-79: z = v1z + a*((w1*dz2) + (w2*dz3))), or -inf.
// Covered samples have w_i >= 0 and w1 + w2 <= O + B (B = b0+b1+b2); hence
// s = fl(fl(w1*dz2) + fl(w2*dz3)) >= (O+B)(m - 3uD) with m = min(0,dz2,dz3),
// D = max|dz|; a = fl(1/o) <= (1+u)/o and (O+B)/o <= 1 + K with K = err/o, so
// q = fl(a*s) >= (1+K)(1+u)^2 (m - 3uD), and z = fl(v1z + q) is monotone in q.
__device__ __forceinline__ float depth_lower_bound(const TriRecord &r, const OrientBound &ob)
{
    if (!depth_bound_usable(r, ob)) return -INFINITY;
    const float K = __fdiv_ru(ob.err, ob.o);
    const float D = fmaxf(fabsf(r.dz2), fabsf(r.dz3));
    const float m = fminf(0.0f, fminf(r.dz2, r.dz3));
    const float mm = __fsub_rd(m, __fmul_ru(kU8, D));                   // m - 8uD
    const float f = __fmul_ru(__fadd_ru(1.0f, K), 1.0f + kU4);          // (1+K)(1+4u)
    const float qlo = __fmul_rd(f, mm);                                 // <= 0
    const float slack = __fadd_ru(__fmul_ru(kU4, __fadd_ru(fabsf(r.v1z), fabsf(qlo))), kTiny);
    return __fsub_rd(__fadd_rd(r.v1z, qlo), slack);
}

// Lower bound of the depths the raster can compute for covered samples inside sample
// rectangle c (one tile's part of a large triangle), or -inf.  The exact
// L(p) = E1(p)*dz2 + E2(p)*dz3 is linear, so its minimum over c is at a corner; at a
// corner, L >= (computed w1*dz2 + w2*dz3, rounded down) - (b1|dz2| + b2|dz3|).  At a
// covered sample s = fl(fl(w1 dz2) + fl(w2 dz3)) >= L(p) - (b1|dz2| + b2|dz3|) -
// 3u(O+B)D, and q = fl(a*s), z = fl(v1z + q) are monotone in s and q.
__device__ __forceinline__ float rect_depth_lower_bound(const TriRecord &r, const OrientBound &ob, const Rect &c)
{
    if (!depth_bound_usable(r, ob)) return -INFINITY;
    const float xs[2] = {(float)c.xa, (float)(c.xb - 1)};
    const float ys[2] = {(float)c.ya, (float)(c.yb - 1)};
    float gmin = INFINITY;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float w1 = edge_eval(r.dx1, r.dy1, r.v3x, r.v3y, xs[i], ys[j]);
            const float w2 = edge_eval(r.dx2, r.dy2, r.v1x, r.v1y, xs[i], ys[j]);
            gmin = fminf(gmin, __fadd_rd(__fmul_rd(w1, r.dz2), __fmul_rd(w2, r.dz3)));
        }
    const float D = fmaxf(fabsf(r.dz2), fabsf(r.dz3));
    const float bz = __fadd_ru(__fmul_ru(ob.eb.b[1], fabsf(r.dz2)), __fmul_ru(ob.eb.b[2], fabsf(r.dz3)));
    const float ob_sum = __fadd_ru(ob.o, ob.err);                           // >= O + B
    const float slack_s = __fadd_ru(__fadd_ru(bz, bz), __fmul_ru(__fmul_ru(kU4, ob_sum), D));
    const float slo = __fsub_rd(gmin, slack_s);
    const float qlo = __fmul_rd(r.a, slo);
    const float slack = __fadd_ru(__fmul_ru(kU4, __fadd_ru(fabsf(r.v1z), fabsf(qlo))), kTiny);
    return __fsub_rd(__fadd_rd(r.v1z, qlo), slack);
}

}  // namespace sloth
