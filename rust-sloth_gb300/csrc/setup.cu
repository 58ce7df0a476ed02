// setup.cu -- vertex transform and per-triangle setup.
//
// Replaces, per triangle, src/rasterizer.rs:56-67 (transform, aabb, sample range,
// a = 1/orient) and src/geometry.rs:37-56 (Triangle::mul/aabb/normal).  The reference
// recomputes utransform*transform per triangle and normal() per covered sample; both
// are the same value every time, so they are formed once (matrix on the host, normal
// here) with the same operation order (record.cuh).
#include <atomic>

#include "bin_common.cuh"
#include "direct.cuh"
#include "record.cuh"
#include "sloth_kernels.h"

namespace sloth {

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

__device__ __forceinline__ Viewport to_vp(const FrameGeom &g)
{
    return Viewport{g.w, g.h, g.image, g.tw, g.th, g.ntx, g.nty, g.pitch};
}

// The three transformed vertices of triangle t, at position p of setup's order.  tv null
// (soups): the thread transforms them itself, which saves the vertex kernel and its round
// trip through memory.
__device__ __forceinline__ void triangle_vertices(const MeshDev &mesh, const float4 *__restrict__ tv, const Mat4 &M,
                                                  uint32_t p, uint32_t t, float4 &p1, float4 &p2, float4 &p3)
{
    uint32_t i1, i2, i3;
    mesh_corners(mesh, p, t, i1, i2, i3);
    if (tv) {
        p1 = __ldg(tv + i1); p2 = __ldg(tv + i2); p3 = __ldg(tv + i3);
    } else {
        p1 = transform_vertex(mesh, M, i1); p2 = transform_vertex(mesh, M, i2); p3 = transform_vertex(mesh, M, i3);
    }
}

// One triangle of the draw with transformed vertices p1, p2, p3 and packed colour rgb
// (live false: none; every lane of the warp calls it for the warp-wide steps): its record,
// its small-triangle tile counts or large-queue slot, and the direct folds of the smallest
// triangles.
template <bool kDirect>
__device__ __forceinline__ void setup_triangle(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                                               const BinBuffers &bb, bool live, uint32_t t, float4 p1, float4 p2,
                                               float4 p3, uint32_t rgb, uint32_t stage)
{
    bool large = false, direct = false;
    TriRecord r;
    TileSpan sp{};
    DirectWalk dw{false, 0, 0u};
    const Viewport vp = to_vp(g);
    if (live) {
        r = build_record(p1, p2, p3, rgb, g.w, g.h, kDirect ? g.direct_max : 0, kDirect ? &dw : nullptr);
        direct = dw.direct;
        if (!direct) sp = tile_span(vp, r);   // a direct triangle is not binned
        store_record(fb.records + tri_base + t, r, sp.ntiles, direct);
        large = sp.large;
    }
    // binning: count tiles of small triangles here and list them for the fill, queue the
    // rest for warps
    const bool binned = live && !large && !direct && sp.ntiles != 0;
    const uint32_t slot1 = count_small_tiles_warp(binned, r, vp, sp, bb.tile_count, bb.tile_cursor);
    if (bb.fill_list) {
        const unsigned bm = __ballot_sync(0xffffffffu, binned);
        if (bm) {
            const int lane = threadIdx.x & 31;
            uint32_t first = 0;
            if (lane == 0) first = atomicAdd(&bb.large_count[2], (uint32_t)__popc(bm));
            first = __shfl_sync(0xffffffffu, first, 0);
            if (binned) bb.fill_list[first + __popc(bm & ((1u << lane) - 1u))] = make_uint2(t, slot1);
        }
    }
    // warp-ballot compaction of the large-triangle queue
    if (__any_sync(0xffffffffu, large)) {
        const int q = large_slot(large, sp.ntiles, bb.large_count, bb.large_cap);
        if (q >= 0) bb.large_queue[q] = t;
    }
    // the smallest triangles fold their samples into the global keys here (direct.cuh)
    if (kDirect && __any_sync(0xffffffffu, direct)) {
        const uint32_t frags = direct_raster_warp(direct, r, tri_base + t, g.w, g.pitch, g.tw,
                                                  reinterpret_cast<unsigned long long *>(fb.keys), dw.xend,
                                                  dw.exit_mask, stage);
        add_frags_warp(frags, fb.fragments);
    }
}

// A block takes tpb triangles, in chunks of setup_chunk(tpb), each in two phases.  Phase 1:
// every triangle gets its sample range and the back-face proof (needs_setup); those with
// nothing to rasterize store their range row and are done, the others are queued in
// shared memory with their vertices and colour.  Phase 2: the queued triangles, dense in
// the lanes, get the rest of their setup (setup_triangle) without touching global memory
// for their inputs again.  Back faces are about half of a closed mesh's triangles, and
// mixed through every warp: without the queue half the lanes of a warp would idle through
// the front faces' work.  kDirect: compiled with the direct path (g.direct_max > 0), which
// needs more registers.  kChunks: compiled for more than one chunk per block (tpb above
// kSetupChunk); the one-chunk form keeps fewer values live through phase 2.
template <bool kDirect, bool kChunks>
__global__ void __launch_bounds__(kSetupThreads, kDirect ? kSetupMinBlocks : kFillMinBlocks)
setup_kernel(MeshDev mesh, const float4 *__restrict__ tv, Mat4 M, uint32_t tri_base, FrameGeom g,
             FrameBuffers fb, BinBuffers bb, int tpb)
{
    __shared__ uint32_t sq_n;
    const uint32_t cap = (uint32_t)setup_chunk(tpb);
    const SetupStash st{cap};
    if (threadIdx.x == 0) sq_n = 0;
    block_sync();
    const uint32_t t0 = blockIdx.x * (uint32_t)tpb, t_end = min(mesh.ntri, t0 + (uint32_t)tpb);
    uint32_t base = 0;
    for (uint32_t c0 = t0; c0 < t_end; c0 += cap) {
        // two triangles per round, their vertex loads issued together (the trip count is
        // the same in every lane: cap is a multiple of twice the block size or equals it)
        // (positions p and q of setup's order: triangles tp and tq; the packed rows are
        // stored by position, everything else by triangle)
        for (uint32_t p = c0 + threadIdx.x; p < c0 + cap; p += 2 * blockDim.x) {
            const uint32_t q = p + blockDim.x;
            const bool lt = p < t_end, lu = q < c0 + cap && q < t_end;
            float4 a1, a2, a3, b1, b2, b3;
            uint32_t ca = 0, cb = 0, tp = 0, tq = 0;
            if (lt) {
                tp = mesh_triangle(mesh, p);
                triangle_vertices(mesh, tv, M, p, tp, a1, a2, a3);
                ca = load_rgb(mesh.rgb, tp);
            }
            if (lu) {
                tq = mesh_triangle(mesh, q);
                triangle_vertices(mesh, tv, M, q, tq, b1, b2, b3);
                cb = load_rgb(mesh.rgb, tq);
            }
            int4 row4;
            const bool kt = lt && needs_setup(a1, a2, a3, g.w, g.h, row4);
            if (lt && !kt) store_row4(fb.records + tri_base + tp, row4);
            if (lt) fb.rows[tri_base + p] = pack_rows(row4.z, row4.w);
            stash_push(st, &sq_n, base, kt, tp, a1, a2, a3, ca);
            const bool ku = lu && needs_setup(b1, b2, b3, g.w, g.h, row4);
            if (lu && !ku) store_row4(fb.records + tri_base + tq, row4);
            if (lu) fb.rows[tri_base + q] = pack_rows(row4.z, row4.w);
            stash_push(st, &sq_n, base, ku, tq, b1, b2, b3, cb);
        }
        block_sync();
        const uint32_t total = sq_n, nq = total - base;
        for (uint32_t q0 = 0; q0 < nq; q0 += blockDim.x) {
            const uint32_t q = q0 + threadIdx.x;
            float4 p1, p2, p3;
            uint32_t rgb = 0, t = 0;
            if (q < nq) t = st.get(q, p1, p2, p3, rgb);
            setup_triangle<kDirect>(tri_base, g, fb, bb, q < nq, t, p1, p2, p3, rgb,
                                    11u * cap + (threadIdx.x >> 5) * (uint32_t)kDirectStageWords);
        }
        if (!kChunks) break;
        base = total;
        if (c0 + cap < t_end) block_sync();   // the next chunk refills the stash
    }
}

// Newline sentinels (src/rasterizer.rs:89-91): in image mode every row y in [y0,y1) of
// every triangle gets frame cell y*w+1 = '\n' after the row's samples.  The resolve needs,
// per row, the last triangle in draw order that wrote it: the maximum draw index whose
// [y0,y1) contains y.  Each triangle folds its interval into a max segment tree with
// O(log h) node updates (canonical decomposition); a row's value is the maximum over its
// leaf-to-root path.  Each block builds a tree for a chunk of triangles in shared memory,
// then merges its non-empty nodes into the frame's tree.  The rows come from the packed
// array setup wrote (4 bytes a triangle, read in setup's order: order maps a position to
// its triangle), not from the records' row 4.
template <bool kShared>
__global__ void __launch_bounds__(1024)
newline_kernel(uint32_t ntri, const uint32_t *__restrict__ order, uint32_t tri_base, uint32_t chunk, FrameGeom g,
               FrameBuffers fb)
{
    extern __shared__ int32_t stree[];
    const int n = g.nl_size;
    int32_t *tree = kShared ? stree : fb.nltree;
    if (kShared) {
        for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) stree[i] = -1;
        block_sync();
    }
    const uint32_t lo = blockIdx.x * chunk, hi = min(ntri, lo + chunk);
    for (uint32_t p = lo + threadIdx.x; p < hi; p += blockDim.x) {
        const int32_t v = (int32_t)(tri_base + (order ? __ldg(order + p) : p));
        const uint32_t yr = __ldg(fb.rows + tri_base + p);
        nltree_update(tree, n, (int)(yr & 0xffffu), (int)(yr >> 16), v, kShared);
    }
    if (kShared) {
        block_sync();
        for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) {
            const int32_t v = stree[i];
            if (v >= 0 && *(volatile int32_t *)&fb.nltree[i] < v) atomicMax(&fb.nltree[i], v);
        }
    }
}

cudaError_t launch_newline(uint32_t ntri, const uint32_t *order, uint32_t tri_base, const FrameGeom &g,
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
        newline_kernel<true><<<blocks, 1024, smem, s>>>(ntri, order, tri_base, chunk, g, fb);
    } else {
        newline_kernel<false><<<blocks, 1024, 0, s>>>(ntri, order, tri_base, chunk, g, fb);
    }
    return cudaGetLastError();
}

// The resets of a frame (device error word, fragment counter, newline tree: frame) and of
// a draw (tile entry counts, large-queue counters: draw) in one launch.
__global__ void __launch_bounds__(256)
frame_reset_kernel(FrameBuffers fb, BinBuffers bb, uint32_t nl_nodes, uint32_t ntiles, int frame, int draw,
                   int tiles_current)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (frame && i < nl_nodes) fb.nltree[i] = -1;
    if (draw && i < ntiles) bb.tile_count[i] = bb.tile_cursor[i] = 0u;
    if (tiles_current && i < ntiles) fb.tile_gen[i] = fb.gen;
    if (i == 0) {
        if (frame) {
            *fb.error = 0u;
            *fb.fragments = 0ull;
        }
        if (draw) bb.large_count[0] = bb.large_count[1] = bb.large_count[2] = 0u;
    }
}

cudaError_t launch_frame_reset(const FrameBuffers &fb, const BinBuffers &bb, uint32_t nl_nodes, uint32_t ntiles,
                               bool frame, bool draw, bool tiles_current, cudaStream_t s)
{
    const uint32_t n = max(frame ? nl_nodes : 1u, (draw || tiles_current) ? ntiles : 1u);
    frame_reset_kernel<<<(n + 255) / 256, 256, 0, s>>>(fb, bb, nl_nodes, ntiles, frame ? 1 : 0, draw ? 1 : 0,
                                                       tiles_current ? 1 : 0);
    return cudaGetLastError();
}

// Keys the samples can write set to the empty key (all bytes 0xff) in a run of tile rows of
// tw cells: the first half of every run of tw keys (key_col: the even columns, all that a
// frame of even width writes).  Two keys per store; n4 = the 16-byte stores, tw >= 8.
__global__ void __launch_bounds__(256) clear_live_keys_kernel(uint4 *keys, uint64_t n4, uint32_t half_shift)
{
    const uint4 empty = make_uint4(~0u, ~0u, ~0u, ~0u);
    const uint64_t mask = (1ull << half_shift) - 1ull;   // stores per half run
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n4; v += (uint64_t)gridDim.x * blockDim.x)
        keys[((v >> half_shift) << (half_shift + 1)) | (v & mask)] = empty;
}

cudaError_t launch_clear_keys(uint64_t *keys, uint64_t ncells, int tw, bool even_width, cudaStream_t s)
{
    if (ncells == 0) return cudaSuccess;
    if (!even_width) return cudaMemsetAsync(keys, 0xff, ncells * sizeof(uint64_t), s);
    uint32_t half_shift = 0;   // log2(tw / 4): 16-byte stores in half a run of tw keys
    while ((4u << half_shift) < (uint32_t)tw) ++half_shift;
    const uint64_t n4 = ncells / 4;   // two keys per store, half of the keys
    uint64_t blocks = (n4 + 255) / 256;
    const uint64_t cap = 16ull * (uint64_t)device_sm_count();
    if (blocks > cap) blocks = cap;
    clear_live_keys_kernel<<<(unsigned)blocks, 256, 0, s>>>(reinterpret_cast<uint4 *>(keys), n4, half_shift);
    return cudaGetLastError();
}

int device_sm_count()
{
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
    if (dev < 64) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
    if (dev < 64) cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

cudaError_t launch_vertex_transform(const MeshDev &mesh, const Mat4 &M, float4 *tv, cudaStream_t s)
{
    if (mesh.nvert == 0) return cudaSuccess;
    const uint32_t quads = (mesh.nvert + 3) / 4;
    vertex_transform_kernel<<<(quads + 255) / 256, 256, 0, s>>>(mesh, M, tv);
    return cudaGetLastError();
}

cudaError_t prepare_setup_kernels()
{
    static std::atomic<uint32_t> done{0};   // devices prepared (bit per device < 32)
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint32_t bit = dev < 32 ? 1u << dev : 0u;
    if (bit && (done.load() & bit)) return cudaSuccess;
    const int bytes = (int)setup_smem_bytes(kMaxTrianglesPerBlock, true);
    if ((e = cudaFuncSetAttribute(setup_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) ||
        (e = cudaFuncSetAttribute(setup_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    done.fetch_or(bit);
    return cudaSuccess;
}

cudaError_t launch_setup(const MeshDev &mesh, const float4 *tv, const Mat4 &M, uint32_t tri_base,
                         const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                         cudaStream_t s, int tpb)
{
    if (mesh.ntri == 0) return cudaSuccess;
    if (!valid_triangles_per_block(tpb)) return cudaErrorInvalidValue;
    const uint32_t blocks = (mesh.ntri + tpb - 1) / tpb;
    const size_t smem = setup_smem_bytes(tpb, g.direct_max > 0);   // prepare_setup_kernels: above 48 KB
    const dim3 grid(blocks), block(setup_block_threads(tpb));
    const bool chunks = tpb > kSetupChunk;
    if (g.direct_max > 0) {
        if (chunks) setup_kernel<true, true><<<grid, block, smem, s>>>(mesh, tv, M, tri_base, g, fb, bb, tpb);
        else setup_kernel<true, false><<<grid, block, smem, s>>>(mesh, tv, M, tri_base, g, fb, bb, tpb);
    } else {
        if (chunks) setup_kernel<false, true><<<grid, block, smem, s>>>(mesh, tv, M, tri_base, g, fb, bb, tpb);
        else setup_kernel<false, false><<<grid, block, smem, s>>>(mesh, tv, M, tri_base, g, fb, bb, tpb);
    }
    return cudaGetLastError();
}

}  // namespace sloth
