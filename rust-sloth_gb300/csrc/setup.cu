// setup.cu -- vertex transform and per-triangle setup.
//
// Replaces, per triangle, src/rasterizer.rs:56-67 (transform, aabb, sample range,
// a = 1/orient) and src/geometry.rs:37-56 (Triangle::mul/aabb/normal).  The reference
// recomputes utransform*transform per triangle and normal() per covered sample; both
// are the same value every time, so they are formed once (matrix on the host, normal
// here) with the same operation order.
#include "bounds.cuh"
#include "sloth_internal.cuh"
#include "sloth_kernels.h"

namespace sloth {

// nalgebra Matrix4*Vector4 with w = 1: ((m0*x + m1*y) + m2*z) + m3*1, each step rounded.
__device__ __forceinline__ float row_dot(const float *m, float x, float y, float z)
{
    float acc = fmul(m[0], x);
    acc = fadd(fmul(m[1], y), acc);
    acc = fadd(fmul(m[2], z), acc);
    acc = fadd(fmul(m[3], 1.0f), acc);
    return acc;
}

// Four vertices per thread: float4 loads of the x, y and z arrays (structure of arrays).
__global__ void __launch_bounds__(256) vertex_transform_kernel(MeshDev mesh, Mat4 M, float4 *tv)
{
    const uint32_t nv = mesh.nvert;
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;   // quad index
    const uint32_t i0 = q * 4;
    if (i0 >= nv) return;
    float xs[4], ys[4], zs[4];
    if (i0 + 4 <= nv) {
        float4 X = __ldg(reinterpret_cast<const float4 *>(mesh.x) + q);
        float4 Y = __ldg(reinterpret_cast<const float4 *>(mesh.y) + q);
        float4 Z = __ldg(reinterpret_cast<const float4 *>(mesh.z) + q);
        xs[0] = X.x; xs[1] = X.y; xs[2] = X.z; xs[3] = X.w;
        ys[0] = Y.x; ys[1] = Y.y; ys[2] = Y.z; ys[3] = Y.w;
        zs[0] = Z.x; zs[1] = Z.y; zs[2] = Z.z; zs[3] = Z.w;
    } else {
        for (int k = 0; k < 4; ++k) {
            uint32_t i = i0 + k < nv ? i0 + k : nv - 1;
            xs[k] = mesh.x[i]; ys[k] = mesh.y[i]; zs[k] = mesh.z[i];
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (i0 + k < nv) {
            float4 o;
            o.x = row_dot(&M.m[0], xs[k], ys[k], zs[k]);
            o.y = row_dot(&M.m[4], xs[k], ys[k], zs[k]);
            o.z = row_dot(&M.m[8], xs[k], ys[k], zs[k]);
            o.w = 0.0f;
            tv[i0 + k] = o;
        }
    }
}

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
__device__ bool right_of_is_empty(const TriRecord &r, int X, int y0, int y1)
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

__device__ __forceinline__ Viewport to_vp(const FrameGeom &g)
{
    return Viewport{g.w, g.h, g.image, g.tw, g.th, g.ntx, g.nty, g.pitch};
}

__global__ void __launch_bounds__(256)
setup_kernel(MeshDev mesh, const float4 *__restrict__ tv, uint32_t tri_base, FrameGeom g,
             FrameBuffers fb, BinBuffers bb)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = t < mesh.ntri;
    bool large = false;
    if (live) {
        uint32_t i1, i2, i3;
        if (mesh.idx) {
            i1 = __ldg(mesh.idx + 3 * (size_t)t + 0);
            i2 = __ldg(mesh.idx + 3 * (size_t)t + 1);
            i3 = __ldg(mesh.idx + 3 * (size_t)t + 2);
        } else {
            i1 = 3 * t + 0; i2 = 3 * t + 1; i3 = 3 * t + 2;
        }
        const float4 p1 = __ldg(tv + i1), p2 = __ldg(tv + i2), p3 = __ldg(tv + i3);
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
        const uint8_t *c = mesh.rgb + 3 * (size_t)t;
        r.rgb = (uint32_t)c[0] | ((uint32_t)c[1] << 8) | ((uint32_t)c[2] << 16);
        // aabb and sample range  (src/geometry.rs:37-42, src/rasterizer.rs:59-66)
        const float mnx = fminf(p1.x, fminf(p2.x, p3.x)), mny = fminf(p1.y, fminf(p2.y, p3.y));
        const float mxx = fmaxf(p1.x, fmaxf(p2.x, p3.x)), mxy = fmaxf(p1.y, fmaxf(p2.y, p3.y));
        r.x0 = sat_lo(ceilf(fmaxf(mnx, 1.0f)), g.w);
        r.y0 = sat_lo(ceilf(fmaxf(mny, 1.0f)), g.h);
        const int x1 = sat_hi(ceilf(fminf(fmul(mxx, 2.0f), (float)(g.w - 1))));
        r.y1 = sat_hi(ceilf(fminf(mxy, (float)(g.h - 1))));
        const float big = 1e18f;
        const bool finite = fabsf(p1.x) < big && fabsf(p1.y) < big && fabsf(p2.x) < big &&
                            fabsf(p2.y) < big && fabsf(p3.x) < big && fabsf(p3.y) < big;
        r.flags = finite ? kFlagFiniteXY : 0u;
        r.xe = x1;
        r.zlo = -INFINITY;
        if (finite && r.x0 < x1 && r.y0 < r.y1) {
            // first column strictly right of the triangle, not left of x0
            const float xf = fadd(floorf(mxx), 1.0f);
            if (xf < (float)x1) {
                const int X = xf <= (float)r.x0 ? r.x0 : (int)xf;
                if (right_of_is_empty(r, X, r.y0, r.y1)) {
                    r.xe = X;
                    r.flags |= kFlagTight;
                }
            }
            // cull triangles that provably cover no sample of the evaluated range (the
            // range right of xe is already proven empty, or xe is the reference's bound)
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
        const uint32_t gtri = tri_base + t;
        fb.records[gtri] = r;

        // binning: count tiles of small triangles here, queue the rest for warps
        const Viewport vp = to_vp(g);
        const TileSpan sp = tile_span(vp, r);
        const Rect &U = sp.U, &W = sp.W, &TU = sp.TU, &TW = sp.TW;
        large = sp.large;
        if (!large) {
            for (int tr = TU.ya; tr < TU.yb; ++tr)
                for (int tc = TU.xa; tc < TU.xb; ++tc)
                    if (tile_hit(r, vp, U, W, tr, tc)) atomicAdd(&bb.tile_count[tr * g.ntx + tc], 1u);
            for (int tr = TW.ya; tr < TW.yb; ++tr)
                for (int tc = TW.xa; tc < TW.xb; ++tc) {
                    if (tr >= TU.ya && tr < TU.yb && tc >= TU.xa && tc < TU.xb) continue;
                    if (tile_hit(r, vp, U, W, tr, tc)) atomicAdd(&bb.tile_count[tr * g.ntx + tc], 1u);
                }
        }
    }
    // warp-ballot compaction of the large-triangle queue
    const unsigned m = __ballot_sync(0xffffffffu, large);
    if (m) {
        const int lane = threadIdx.x & 31;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(bb.large_count, (uint32_t)__popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (large) bb.large_queue[base + __popc(m & ((1u << lane) - 1u))] = t;
    }
}

// Newline sentinels (src/rasterizer.rs:89-91): in image mode every row y in [y0,y1) of
// every triangle gets frame cell y*w+1 = '\n' after the row's samples.  The resolve needs,
// per row, the last triangle in draw order that wrote it: the maximum draw index whose
// [y0,y1) contains y.  Each triangle folds its interval into a max segment tree with
// O(log h) node updates (canonical decomposition); a row's value is the maximum over its
// leaf-to-root path.  Each block builds a tree for a chunk of triangles in shared memory,
// then merges its non-empty nodes into the frame's tree.
template <bool kShared>
__global__ void __launch_bounds__(1024)
newline_kernel(uint32_t ntri, uint32_t tri_base, uint32_t chunk, FrameGeom g, FrameBuffers fb)
{
    extern __shared__ int32_t stree[];
    const int n = g.nl_size;
    int32_t *tree = kShared ? stree : fb.nltree;
    if (kShared) {
        for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) stree[i] = -1;
        __syncthreads();
    }
    const uint32_t lo = blockIdx.x * chunk, hi = min(ntri, lo + chunk);
    for (uint32_t t = lo + threadIdx.x; t < hi; t += blockDim.x) {
        const int32_t v = (int32_t)(tri_base + t);
        const int4 yr = __ldg(reinterpret_cast<const int4 *>(fb.records + tri_base + t) + 4);
        int l = yr.z + n, r = yr.w + n;   // [y0, y1)
        while (l < r) {
            if (l & 1) {
                if (kShared || *(volatile int32_t *)&tree[l] < v) atomicMax(&tree[l], v);
                ++l;
            }
            if (r & 1) {
                --r;
                if (kShared || *(volatile int32_t *)&tree[r] < v) atomicMax(&tree[r], v);
            }
            l >>= 1;
            r >>= 1;
        }
    }
    if (kShared) {
        __syncthreads();
        for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) {
            const int32_t v = stree[i];
            if (v >= 0 && *(volatile int32_t *)&fb.nltree[i] < v) atomicMax(&fb.nltree[i], v);
        }
    }
}

cudaError_t launch_newline(uint32_t ntri, uint32_t tri_base, const FrameGeom &g,
                           const FrameBuffers &fb, cudaStream_t s)
{
    if (ntri == 0 || !g.image) return cudaSuccess;
    const uint32_t chunk = 8192;
    const uint32_t blocks = (ntri + chunk - 1) / chunk;
    const size_t smem = 2 * (size_t)g.nl_size * sizeof(int32_t);
    if (smem <= 128 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(newline_kernel<true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, 128 * 1024);
        if (e != cudaSuccess) return e;
        newline_kernel<true><<<blocks, 1024, smem, s>>>(ntri, tri_base, chunk, g, fb);
    } else {
        newline_kernel<false><<<blocks, 1024, 0, s>>>(ntri, tri_base, chunk, g, fb);
    }
    return cudaGetLastError();
}

cudaError_t launch_vertex_transform(const MeshDev &mesh, const Mat4 &M, float4 *tv, cudaStream_t s)
{
    if (mesh.nvert == 0) return cudaSuccess;
    const uint32_t quads = (mesh.nvert + 3) / 4;
    vertex_transform_kernel<<<(quads + 255) / 256, 256, 0, s>>>(mesh, M, tv);
    return cudaGetLastError();
}

cudaError_t launch_setup(const MeshDev &mesh, const float4 *tv, uint32_t tri_base,
                         const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                         cudaStream_t s)
{
    if (mesh.ntri == 0) return cudaSuccess;
    setup_kernel<<<(mesh.ntri + 255) / 256, 256, 0, s>>>(mesh, tv, tri_base, g, fb, bb);
    return cudaGetLastError();
}

}  // namespace sloth
