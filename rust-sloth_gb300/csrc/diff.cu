// diff.cu -- differentiable shading of a rendered batch and its hand-written adjoint.
//
// There is no counterpart in the reference: sloth only picks a character from the
// screen-space normal's z (src/rasterizer.rs:76).  The image defined here reduces to that
// quantity: for the winning sample (x, y) of a depth cell (the render's visibility, held
// fixed) and its triangle A, B, C in screen space,
//     rgb = (b0*c(A) + b1*c(B) + b2*c(C)) * clamp(n_hat . L, 0, 1)
// with b_i = w_i / orient(A,B,C) the barycentric weights of (x, y), c the f32 vertex
// colours, n_hat = unit((B-A) x (C-A)) and L the light direction in screen space; with
// L = (0,0,1) the shade factor is the reference's normal z.
//
// The backward pass walks samples (x, y) rather than cells, so that the lanes of a warp
// hold consecutive samples of one row: their winners are mostly runs of one triangle,
// which a segmented warp reduction folds into one set of atomics per run.  The head lane
// of a run maps the screen-space position gradients to object space through the draw's
// matrix (object = M3^T * screen; the vertex transform has no divide) and adds them, and
// the colour gradients, to the mesh's vertices.  The light gradient is reduced per block.
#include "diff_kernels.h"
#include "resolve_common.cuh"

namespace sloth {

namespace {

constexpr uint32_t kNoTri = 0xffffffffu;
constexpr int kDiffThreads = 256;

struct Hit {
    uint32_t tri;      // frame-local triangle (draw order), kNoTri when none
    int32_t x, y;      // sample point
};

// Winning sample of depth cell id of frame f, decoded from its depth key.
__device__ __forceinline__ Hit hit_from_key(const BatchFrame &f, uint64_t id)
{
    const int r = (int)(id / f.g.w), cc = (int)(id - (uint64_t)r * f.g.w);
    const uint64_t key = key_at(f.g, f.fb, r, cc);
    if (key == kEmptyKey) return Hit{kNoTri, 0, 0};
    const uint32_t lo = (uint32_t)key;
    if (lo & 1u) return Hit{lo >> 1, cc >> 1, r};
    return Hit{lo >> 1, (cc + f.g.w) >> 1, r - 1};
}

__device__ __forceinline__ uint2 pack_hit(const Hit &h)
{
    return make_uint2(h.tri, (uint32_t)h.x | ((uint32_t)h.y << 16));
}

__device__ __forceinline__ Hit unpack_hit(uint2 v)
{
    return Hit{v.x, (int32_t)(v.y & 0xffffu), (int32_t)(v.y >> 16)};
}

// The draw of frame-local triangle `tri`: the last of the frame's draws whose first
// triangle is <= tri.
__device__ __forceinline__ uint32_t draw_of(const BatchDev &b, const BatchFrame &f, uint32_t tri)
{
    uint32_t lo = f.first_draw, hi = f.first_draw + f.ndraws - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (b.draws[mid].local_base <= tri) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

struct Tri {
    float3 A, B, C;
    uint32_t i0, i1, i2;   // mesh vertex ids
};

__device__ __forceinline__ Tri load_tri(const BatchDev &b, const BatchDraw &d, uint32_t t)
{
    Tri g;
    if (d.mesh.idx) {
        g.i0 = __ldg(d.mesh.idx + 3 * (size_t)t);
        g.i1 = __ldg(d.mesh.idx + 3 * (size_t)t + 1);
        g.i2 = __ldg(d.mesh.idx + 3 * (size_t)t + 2);
    } else {
        g.i0 = 3 * t;
        g.i1 = 3 * t + 1;
        g.i2 = 3 * t + 2;
    }
    const float4 *tv = b.tv + d.vert_off;
    const float4 a = tv[g.i0], bb = tv[g.i1], c = tv[g.i2];
    g.A = make_float3(a.x, a.y, a.z);
    g.B = make_float3(bb.x, bb.y, bb.z);
    g.C = make_float3(c.x, c.y, c.z);
    return g;
}

__device__ __forceinline__ float orient2(float ax, float ay, float bx, float by, float cx, float cy)
{
    return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
}
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 ld3(const float *p)
{
    return make_float3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

struct Shade {
    bool ok;                 // non-degenerate triangle
    float b0, b1, b2, o;     // barycentrics, orient(A,B,C)
    float3 c0, c1, c2;       // vertex colours
    float3 col;              // interpolated colour
    float3 nhat;
    float nlen, ndl, s;      // |n|, n_hat . L, clamp(n_hat . L, 0, 1)
};

__device__ __forceinline__ Shade shade_at(const Tri &g, float px, float py, const float *vrgb, float3 L)
{
    Shade e;
    e.o = orient2(g.A.x, g.A.y, g.B.x, g.B.y, g.C.x, g.C.y);
    const float3 n = cross3(sub3(g.B, g.A), sub3(g.C, g.A));
    e.nlen = sqrtf(dot3(n, n));
    e.ok = e.o != 0.0f && e.nlen > 0.0f && isfinite(e.o) && isfinite(e.nlen);
    if (!e.ok) return e;
    const float io = 1.0f / e.o;
    e.b0 = orient2(g.B.x, g.B.y, g.C.x, g.C.y, px, py) * io;
    e.b1 = orient2(g.C.x, g.C.y, g.A.x, g.A.y, px, py) * io;
    e.b2 = orient2(g.A.x, g.A.y, g.B.x, g.B.y, px, py) * io;
    e.c0 = ld3(vrgb + 3 * (size_t)g.i0);
    e.c1 = ld3(vrgb + 3 * (size_t)g.i1);
    e.c2 = ld3(vrgb + 3 * (size_t)g.i2);
    e.col = make_float3(e.b0 * e.c0.x + e.b1 * e.c1.x + e.b2 * e.c2.x, e.b0 * e.c0.y + e.b1 * e.c1.y + e.b2 * e.c2.y,
                        e.b0 * e.c0.z + e.b1 * e.c1.z + e.b2 * e.c2.z);
    const float il = 1.0f / e.nlen;
    e.nhat = make_float3(n.x * il, n.y * il, n.z * il);
    e.ndl = dot3(e.nhat, L);
    e.s = fminf(fmaxf(e.ndl, 0.0f), 1.0f);
    return e;
}

__global__ void __launch_bounds__(kDiffThreads)
batch_shade_kernel(BatchDev b, const int2 *__restrict__ blocks, const float *__restrict__ vrgb,
                   const float *__restrict__ light, float *__restrict__ rgb, uint2 *__restrict__ vis)
{
    const int2 blk = blocks[blockIdx.x];
    const BatchFrame &f = b.frames[blk.x];
    const uint64_t nz = (uint64_t)f.g.w * f.g.h;
    const uint64_t end = min(nz, (uint64_t)blk.y + kDiffChunk);
    const float3 L = ld3(light);
    for (uint64_t c = (uint64_t)blk.y + threadIdx.x; c < end; c += kDiffThreads) {
        const uint64_t gc = f.z_off + c;
        const Hit h = hit_from_key(f, c);
        float3 out = make_float3(0.0f, 0.0f, 0.0f);
        if (h.tri != kNoTri) {
            const BatchDraw &d = b.draws[draw_of(b, f, h.tri)];
            const Tri g = load_tri(b, d, h.tri - d.local_base);
            const Shade e = shade_at(g, (float)h.x, (float)h.y, vrgb, L);
            if (e.ok) out = make_float3(e.col.x * e.s, e.col.y * e.s, e.col.z * e.s);
        }
        if (vis) vis[gc] = pack_hit(h);
        rgb[3 * gc + 0] = out.x;
        rgb[3 * gc + 1] = out.y;
        rgb[3 * gc + 2] = out.z;
    }
}

// v summed over the lanes [lane, seg_end) of the caller's run (all 32 lanes call).
__device__ __forceinline__ float run_sum(float v, int lane, int seg_end)
{
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const float o = __shfl_down_sync(0xffffffffu, v, d);
        if (lane + d < seg_end) v += o;
    }
    return v;
}

__global__ void __launch_bounds__(kDiffThreads)
batch_shade_backward_kernel(BatchDev b, const int2 *__restrict__ blocks, const float *__restrict__ vrgb,
                            const float *__restrict__ light, const float *__restrict__ grad_rgb,
                            const uint2 *__restrict__ vis, float *__restrict__ gpos, float *__restrict__ gcol,
                            float *__restrict__ glight)
{
    __shared__ float sl[3][kDiffThreads / 32];
    const int2 blk = blocks[blockIdx.x];
    const BatchFrame &f = b.frames[blk.x];
    const int w = f.g.w;
    const uint64_t nz = (uint64_t)w * f.g.h;
    const float3 L = ld3(light);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float gl0 = 0.0f, gl1 = 0.0f, gl2 = 0.0f;
    // warp-uniform trip count: every lane takes part in the run reductions
    for (uint32_t i = threadIdx.x; i < kDiffChunk; i += kDiffThreads) {
        const uint64_t smp = (uint64_t)blk.y + i;            // sample index y*w + x
        uint32_t tri = kNoTri, draw = 0;
        int x = 0, y = 0;
        if (smp < nz) {
            y = (int)(smp / w);
            x = (int)(smp - (uint64_t)y * w);
            const uint64_t id = (uint64_t)y * w + 2 * (uint64_t)x;
            if (id < nz) {
                const Hit h = vis ? unpack_hit(vis[f.z_off + id]) : hit_from_key(f, id);
                if (h.tri != kNoTri && h.x == x && h.y == y) tri = h.tri;
            }
        }
        float v[18];
#pragma unroll
        for (int k = 0; k < 18; ++k) v[k] = 0.0f;
        Tri g{};
        if (tri != kNoTri) {
            draw = draw_of(b, f, tri);
            const BatchDraw &d = b.draws[draw];
            g = load_tri(b, d, tri - d.local_base);
            const float px = (float)x, py = (float)y;
            const Shade e = shade_at(g, px, py, vrgb, L);
            const uint64_t gc = f.z_off + (uint64_t)y * w + 2 * (uint64_t)x;
            const float3 go = ld3(grad_rgb + 3 * gc);
            if (e.ok && (go.x != 0.0f || go.y != 0.0f || go.z != 0.0f)) {
                // rgb = col * s
                const float3 gc3 = make_float3(go.x * e.s, go.y * e.s, go.z * e.s);
                const float gs = (e.ndl > 0.0f && e.ndl < 1.0f) ? dot3(go, e.col) : 0.0f;
                // colour: d col / d c_i = b_i
                v[9] = gc3.x * e.b0;  v[10] = gc3.y * e.b0; v[11] = gc3.z * e.b0;
                v[12] = gc3.x * e.b1; v[13] = gc3.y * e.b1; v[14] = gc3.z * e.b1;
                v[15] = gc3.x * e.b2; v[16] = gc3.y * e.b2; v[17] = gc3.z * e.b2;
                // barycentrics: b_i = w_i / o, d b_i = (d w_i - b_i d o) / o
                const float gb0 = dot3(gc3, e.c0), gb1 = dot3(gc3, e.c1), gb2 = dot3(gc3, e.c2);
                const float io = 1.0f / e.o;
                const float k = gb0 * e.b0 + gb1 * e.b1 + gb2 * e.b2;
                const float3 A = g.A, B = g.B, C = g.C;
                v[0] = io * (gb1 * (py - C.y) + gb2 * (B.y - py) - k * (B.y - C.y));
                v[1] = io * (gb1 * (C.x - px) + gb2 * (px - B.x) - k * (C.x - B.x));
                v[3] = io * (gb0 * (C.y - py) + gb2 * (py - A.y) - k * (C.y - A.y));
                v[4] = io * (gb0 * (px - C.x) + gb2 * (A.x - px) - k * (A.x - C.x));
                v[6] = io * (gb0 * (py - B.y) + gb1 * (A.y - py) - k * (A.y - B.y));
                v[7] = io * (gb0 * (B.x - px) + gb1 * (px - A.x) - k * (B.x - A.x));
                if (gs != 0.0f) {
                    // s = n_hat . L, n_hat = n / |n|, n = (B-A) x (C-A)
                    const float il = 1.0f / e.nlen;
                    const float3 gn = make_float3(gs * (L.x - e.ndl * e.nhat.x) * il, gs * (L.y - e.ndl * e.nhat.y) * il,
                                                  gs * (L.z - e.ndl * e.nhat.z) * il);
                    const float3 e1 = sub3(B, A), e2 = sub3(C, A);
                    const float3 ge1 = cross3(e2, gn), ge2 = cross3(gn, e1);
                    v[3] += ge1.x; v[4] += ge1.y; v[5] += ge1.z;
                    v[6] += ge2.x; v[7] += ge2.y; v[8] += ge2.z;
                    v[0] -= ge1.x + ge2.x; v[1] -= ge1.y + ge2.y; v[2] -= ge1.z + ge2.z;
                    gl0 += gs * e.nhat.x;
                    gl1 += gs * e.nhat.y;
                    gl2 += gs * e.nhat.z;
                }
            }
        }
        // runs of equal (frame, triangle) over consecutive lanes
        const uint32_t slot = tri == kNoTri ? kNoTri : f.rec_off + tri;
        const uint32_t prev = __shfl_up_sync(0xffffffffu, slot, 1);
        const bool head = lane == 0 || prev != slot;
        const unsigned heads = __ballot_sync(0xffffffffu, head);
        const unsigned above = lane == 31 ? 0u : (heads & ~((2u << lane) - 1u));
        const int seg_end = above ? __ffs(above) - 1 : 32;
#pragma unroll
        for (int k = 0; k < 18; ++k) v[k] = run_sum(v[k], lane, seg_end);
        if (head && tri != kNoTri) {
            const Mat4 &M = b.mats[draw];
            const uint32_t ids[3] = {g.i0, g.i1, g.i2};
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float sx = v[3 * q], sy = v[3 * q + 1], sz = v[3 * q + 2];
                if (gpos && (sx != 0.0f || sy != 0.0f || sz != 0.0f)) {
#pragma unroll
                    for (int j = 0; j < 3; ++j)
                        atomicAdd(gpos + 3 * (size_t)ids[q] + j, M.m[j] * sx + M.m[4 + j] * sy + M.m[8 + j] * sz);
                }
                if (gcol) {
#pragma unroll
                    for (int j = 0; j < 3; ++j)
                        if (v[9 + 3 * q + j] != 0.0f) atomicAdd(gcol + 3 * (size_t)ids[q] + j, v[9 + 3 * q + j]);
                }
            }
        }
    }
#pragma unroll
    for (int dd = 16; dd > 0; dd >>= 1) {
        gl0 += __shfl_xor_sync(0xffffffffu, gl0, dd);
        gl1 += __shfl_xor_sync(0xffffffffu, gl1, dd);
        gl2 += __shfl_xor_sync(0xffffffffu, gl2, dd);
    }
    if (lane == 0) {
        sl[0][wid] = gl0;
        sl[1][wid] = gl1;
        sl[2][wid] = gl2;
    }
    block_sync();
    if (glight && threadIdx.x < 3) {
        float s = 0.0f;
        for (int q = 0; q < kDiffThreads / 32; ++q) s += sl[threadIdx.x][q];
        if (s != 0.0f) atomicAdd(glight + threadIdx.x, s);
    }
}

}  // namespace

cudaError_t launch_batch_shade(const BatchDev &b, const int2 *blocks, uint32_t nblocks, const float *vrgb,
                               const float *light, float *rgb, uint2 *vis, cudaStream_t s)
{
    if (!nblocks) return cudaSuccess;
    batch_shade_kernel<<<nblocks, kDiffThreads, 0, s>>>(b, blocks, vrgb, light, rgb, vis);
    return cudaGetLastError();
}

cudaError_t launch_batch_shade_backward(const BatchDev &b, const int2 *blocks, uint32_t nblocks, const float *vrgb,
                                        const float *light, const float *grad_rgb, const uint2 *vis, float *gpos,
                                        float *gcol, float *glight, cudaStream_t s)
{
    if (!nblocks) return cudaSuccess;
    batch_shade_backward_kernel<<<nblocks, kDiffThreads, 0, s>>>(b, blocks, vrgb, light, grad_rgb, vis, gpos, gcol,
                                                                 glight);
    return cudaGetLastError();
}

}  // namespace sloth
