// batch.cu -- kernels of the batched path: many frames (views, meshes, viewports) in one
// pass of each stage, and one persistent raster kernel over a device-side (frame, tile)
// work queue.  Every per-triangle, per-tile and per-cell step is the single-frame one
// (record.cuh, bin_common.cuh, raster_common.cuh, resolve_common.cuh) applied to the
// item's frame, so each frame is bit-identical to drawing it alone.
#include "batch_kernels.h"
#include "bin_common.cuh"
#include "direct.cuh"
#include "raster_common.cuh"
#include "record.cuh"
#include "resolve_common.cuh"

namespace sloth {

__device__ __forceinline__ Viewport vp_batch(const FrameGeom &g)
{
    return Viewport{g.w, g.h, g.image, g.tw, g.th, g.ntx, g.nty, g.pitch};
}

// blocks[i] = (draw, first vertex quad): four vertices per thread, float4 SoA loads.
__global__ void __launch_bounds__(256) batch_vertex_kernel(BatchDev b, const int2 *__restrict__ blocks)
{
    const int2 blk = blocks[blockIdx.x];
    const BatchDraw &d = b.draws[blk.x];
    const Mat4 M = b.mats[blk.x];
    const uint32_t nv = d.mesh.nvert;
    const uint32_t q = (uint32_t)blk.y + threadIdx.x;
    const uint32_t i0 = q * 4;
    if (i0 >= nv) return;
    float xs[4], ys[4], zs[4];
    if (i0 + 4 <= nv) {
        const float4 X = __ldg(reinterpret_cast<const float4 *>(d.mesh.x) + q);
        const float4 Y = __ldg(reinterpret_cast<const float4 *>(d.mesh.y) + q);
        const float4 Z = __ldg(reinterpret_cast<const float4 *>(d.mesh.z) + q);
        xs[0] = X.x; xs[1] = X.y; xs[2] = X.z; xs[3] = X.w;
        ys[0] = Y.x; ys[1] = Y.y; ys[2] = Y.z; ys[3] = Y.w;
        zs[0] = Z.x; zs[1] = Z.y; zs[2] = Z.z; zs[3] = Z.w;
    } else {
        for (int k = 0; k < 4; ++k) {
            const uint32_t i = i0 + k < nv ? i0 + k : nv - 1;
            xs[k] = d.mesh.x[i]; ys[k] = d.mesh.y[i]; zs[k] = d.mesh.z[i];
        }
    }
    float4 *tv = b.tv + d.vert_off;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (i0 + k < nv)
            tv[i0 + k] = make_float4(row_dot(&M.m[0], xs[k], ys[k], zs[k]), row_dot(&M.m[4], xs[k], ys[k], zs[k]),
                                     row_dot(&M.m[8], xs[k], ys[k], zs[k]), 0.0f);
}

// The three vertices of triangle t of draw d, at position p of setup's order of the mesh,
// transformed by the draw's matrix M in place (the vertex kernel's operations): a mesh
// shared by many views stays in L2, and no transformed-vertex buffer is written and read
// back for the render.
__device__ __forceinline__ void batch_triangle_vertices(const BatchDraw &d, const Mat4 &M, uint32_t p, uint32_t t,
                                                        float4 &p1, float4 &p2, float4 &p3)
{
    uint32_t i1, i2, i3;
    mesh_corners(d.mesh, p, t, i1, i2, i3);
    p1 = transform_vertex(d.mesh, M, i1);
    p2 = transform_vertex(d.mesh, M, i2);
    p3 = transform_vertex(d.mesh, M, i3);
}

// One triangle t of draw d with transformed vertices p1, p2, p3 and packed colour rgb
// (live false: none; every lane of the warp calls it): record, small-triangle tile
// counts, fill list or large queue, and the direct folds of the smallest triangles.
template <bool kDirect>
__device__ __forceinline__ void batch_setup_triangle(const BatchDev &b, const BatchDraw &d, const BatchFrame &f,
                                                     bool live, uint32_t t, float4 p1, float4 p2, float4 p3,
                                                     uint32_t rgb, uint32_t stage)
{
    bool large = false, direct = false;
    DirectWalk dw{false, 0, 0u};
    TriRecord r;
    TileSpan sp{};
    const Viewport vp = vp_batch(f.g);
    if (live) {
        r = build_record(p1, p2, p3, rgb, f.g.w, f.g.h, kDirect ? f.g.direct_max : 0, kDirect ? &dw : nullptr);
        direct = dw.direct;
        if (!direct) sp = tile_span(vp, r);   // a direct triangle is not binned
        // a triangle with nothing to rasterize is never read back here (the fill walks the
        // fill list, the newline the packed rows): its record is not written
        if (direct || sp.ntiles != 0) store_record(f.fb.records + d.local_base + t, r, sp.ntiles, direct);
        large = sp.large;
    }
    const bool binned = live && !large && !direct && sp.ntiles != 0;
    const uint32_t slot1 = count_small_tiles_warp(binned, r, vp, sp, b.bb.tile_count + f.tile_off,
                                                  b.bb.tile_cursor + f.tile_off);
    // the fill's work list: one atomic per warp
    const unsigned bm = __ballot_sync(0xffffffffu, binned);
    if (bm) {
        const int lane = threadIdx.x & 31;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(b.fill_count, (uint32_t)__popc(bm));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (binned) b.fill_list[base + __popc(bm & ((1u << lane) - 1u))] = make_uint4(d.frame, d.local_base + t, slot1, 0u);
    }
    if (__any_sync(0xffffffffu, large)) {
        const int q = large_slot(large, sp.ntiles, b.bb.large_count, b.bb.large_cap);
        if (q >= 0) {
            b.bb.large_queue[q] = d.local_base + t;   // frame-local draw index
            b.large_frame[q] = d.frame;
        }
    }
    // the smallest triangles fold their samples into the frame's global keys (direct.cuh)
    if (kDirect && __any_sync(0xffffffffu, direct)) {
        const uint32_t frags = direct_raster_warp(direct, r, d.local_base + t, f.g.w, f.g.pitch, f.g.tw,
                                                  reinterpret_cast<unsigned long long *>(f.fb.keys), dw.xend,
                                                  dw.exit_mask, stage);
        add_frags_warp(frags, f.fb.fragments);
    }
}

// blocks[i] = (draw, first triangle): b.tpb triangles of the draw in the single-frame
// setup's chunks and two phases (setup.cu): the range and the back-face proof for every
// triangle, the rest of the setup for the ones queued in shared memory with their vertices.
template <bool kDirect, bool kChunks>
__global__ void __launch_bounds__(kSetupThreads, kDirect ? kSetupMinBlocks : kFillMinBlocks) batch_setup_kernel(BatchDev b, const int2 *__restrict__ blocks)
{
    __shared__ uint32_t sq_n;
    // the draw's and frame's descriptors in shared memory: read there, their fields are not
    // reloaded from global memory after each of the block's record stores
    __shared__ BatchDraw sd;
    __shared__ BatchFrame sf;
    __shared__ Mat4 sm;
    const int2 blk = blocks[blockIdx.x];
    if (threadIdx.x < 16) sm.m[threadIdx.x] = b.mats[blk.x].m[threadIdx.x];
    const uint32_t cap = (uint32_t)setup_chunk(b.tpb);
    const SetupStash st{cap};
    if (threadIdx.x == 0) {
        sq_n = 0;
        sd = b.draws[blk.x];
        sf = b.frames[sd.frame];
    }
    block_sync();
    const BatchDraw &d = sd;
    const BatchFrame &f = sf;
    const uint32_t t0 = (uint32_t)blk.y, t_end = min(d.mesh.ntri, t0 + (uint32_t)b.tpb);
    uint32_t base = 0;
    for (uint32_t c0 = t0; c0 < t_end; c0 += cap) {
        // two triangles per round, their vertex loads issued together (the same trip count
        // in every lane)
        // (positions p and q of setup's order: triangles tp and tq; the packed rows are
        // stored by position, everything else by triangle)
        for (uint32_t p = c0 + threadIdx.x; p < c0 + cap; p += 2 * blockDim.x) {
            const uint32_t q = p + blockDim.x;
            const bool lt = p < t_end, lu = q < c0 + cap && q < t_end;
            float4 a1, a2, a3, b1, b2, b3;
            uint32_t ca = 0, cb = 0, tp = 0, tq = 0;
            if (lt) {
                tp = mesh_triangle(d.mesh, p);
                batch_triangle_vertices(d, sm, p, tp, a1, a2, a3);
                ca = load_rgb(d.mesh.rgb, tp);
            }
            if (lu) {
                tq = mesh_triangle(d.mesh, q);
                batch_triangle_vertices(d, sm, q, tq, b1, b2, b3);
                cb = load_rgb(d.mesh.rgb, tq);
            }
            int4 row4;
            const bool kt = lt && needs_setup(a1, a2, a3, f.g.w, f.g.h, row4);
            if (lt) f.fb.rows[d.local_base + p] = pack_rows(row4.z, row4.w);
            stash_push(st, &sq_n, base, kt, tp, a1, a2, a3, ca);
            const bool ku = lu && needs_setup(b1, b2, b3, f.g.w, f.g.h, row4);
            if (lu) f.fb.rows[d.local_base + q] = pack_rows(row4.z, row4.w);
            stash_push(st, &sq_n, base, ku, tq, b1, b2, b3, cb);
        }
        block_sync();
        const uint32_t total = sq_n, nq = total - base;
        for (uint32_t q0 = 0; q0 < nq; q0 += blockDim.x) {
            const uint32_t q = q0 + threadIdx.x;
            float4 p1, p2, p3;
            uint32_t rgb = 0, t = 0;
            if (q < nq) t = st.get(q, p1, p2, p3, rgb);
            batch_setup_triangle<kDirect>(b, d, f, q < nq, t, p1, p2, p3, rgb,
                                          11u * cap + (threadIdx.x >> 5) * (uint32_t)kDirectStageWords);
        }
        if (!kChunks) break;
        base = total;
        if (c0 + cap < t_end) block_sync();   // the next chunk refills the stash
    }
}

// blocks[i] = (draw, first triangle of a chunk): newline segment tree of the draw's frame.
template <bool kShared>
__global__ void __launch_bounds__(1024) batch_newline_kernel(BatchDev b, const int2 *__restrict__ blocks)
{
    extern __shared__ int32_t stree[];
    const int2 blk = blocks[blockIdx.x];
    const BatchDraw &d = b.draws[blk.x];
    const BatchFrame &f = b.frames[d.frame];
    if (!f.g.image) return;
    const int n = f.g.nl_size;
    int32_t *tree = kShared ? stree : f.fb.nltree;
    if (kShared) {
        for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) stree[i] = -1;
        block_sync();
    }
    const uint32_t lo = (uint32_t)blk.y, hi = min(d.mesh.ntri, lo + kBatchNewlineChunk);
    for (uint32_t p = lo + threadIdx.x; p < hi; p += blockDim.x) {
        const int32_t v = (int32_t)(d.local_base + mesh_triangle(d.mesh, p));
        const uint32_t yr = __ldg(f.fb.rows + d.local_base + p);
        nltree_update(tree, n, (int)(yr & 0xffffu), (int)(yr >> 16), v, kShared);
    }
    if (kShared) {
        block_sync();
        for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) {
            const int32_t v = stree[i];
            if (v >= 0 && *(volatile int32_t *)&f.fb.nltree[i] < v) atomicMax(&f.fb.nltree[i], v);
        }
    }
}

// One warp per queued large triangle, any frame.
template <bool kFill>
__global__ void __launch_bounds__(256) batch_bin_large_kernel(BatchDev b)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t items = large_items(b.bb.large_count);
    for (uint32_t it = warp; it < items; it += nwarps) {
        uint32_t q, part, nparts;
        if (!large_item(it, b.bb.large_count, b.bb.large_cap, q, part, nparts)) break;
        const BatchFrame &f = b.frames[b.large_frame[q]];
        const uint32_t gtri = b.bb.large_queue[q];
        bin_large_warp<kFill>(f.fb.records + gtri, gtri, vp_batch(f.g), b.bb.tile_count + f.tile_off,
                              b.bb.tile_cursor + f.tile_off, b.bb.entries, b.bb.capacity, lane, part, nparts);
    }
}

// The small binned triangles setup listed, 256 per block and round (grid-stride): their
// tile entries.  A warp's lanes may hold triangles of different frames; their tiles are
// global tile indices.
__global__ void __launch_bounds__(kSetupThreads, kFillMinBlocks) batch_fill_kernel(BatchDev b)
{
    const uint32_t n = *b.fill_count;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool live = i < n;
        const uint4 e = live ? b.fill_list[i] : make_uint4(0u, 0u, 0u, 0u);
        const BatchFrame &f = b.frames[e.x];
        const Viewport vp = vp_batch(f.g);
        TriRecord r;
        TileSpan sp{};
        if (live) {
            r = load_record(f.fb.records, e.y);
            sp = tile_span(vp, r);
        }
        fill_small_warp(live, r, e.y, vp, sp, b.bb.tile_offset, b.bb.tile_cursor, b.bb.entries, b.bb.capacity, e.z,
                        f.tile_off);
    }
}

__device__ __forceinline__ uint32_t frame_of_tile(const BatchDev &b, uint32_t tile)
{
    // last frame whose first tile is <= tile
    uint32_t lo = 0, hi = b.nframes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (b.frame_tile_off[mid] <= tile) lo = mid;
        else hi = mid;
    }
    return lo;
}

// One thread per global tile: the tile's raster items (tile, slice); a tile rasterized in
// slices gets its keys cleared and its generation set first (bin_items_kernel, per frame).
__global__ void __launch_bounds__(256) batch_items_kernel(BatchDev b)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) *b.queue = 0u;   // the persistent raster's item counter
    if (t >= b.total_tiles) return;
    const uint32_t nt = b.total_tiles;
    const SplitParams sp{b.bb.slice_offset[nt + 1], b.bb.slice_offset[nt + 2]};
    const uint32_t cnt = b.bb.tile_count[t], ns = tile_slices(cnt, sp);
    const bool split = cnt > sp.threshold;
    const uint32_t off = item_offset(b.bb.slice_offset, nt, t, cnt, sp.threshold);
    for (uint32_t k = 0; k < ns && off + k < b.bb.item_capacity; ++k) b.bb.items[off + k] = make_uint2(t, k);
    if (split) {
        const BatchFrame &f = b.frames[frame_of_tile(b, t)];
        const uint32_t lt = t - f.tile_off;
        if (f.fb.tile_gen[lt] != f.fb.gen) {
            const int tr = (int)lt / f.g.ntx, tc = (int)lt - tr * f.g.ntx;
            unsigned long long *k0 = reinterpret_cast<unsigned long long *>(f.fb.keys) +
                                     (size_t)tr * f.g.th * f.g.pitch + (size_t)tc * f.g.tw;
            for (int r = 0; r < f.g.th; ++r)
                for (int c = 0; c < live_keys_per_row(f.g.w, f.g.tw); ++c) k0[(size_t)r * f.g.pitch + c] = kEmptyKey;
            f.fb.tile_gen[lt] = f.fb.gen;
        }
    }
}

// Raster item i (a tile, or a slice of a split tile, of any frame) of the item list built by
// batch_items_kernel; false when its key load gave up (raster_tile).
template <int TW, int TH>
__device__ __forceinline__ bool batch_raster_item(TileSmem<TW, TH> &S, const BatchDev &b, uint32_t i, uint32_t &phase)
{
    const uint2 it = b.bb.items[i];
    const BatchFrame &f = b.frames[frame_of_tile(b, it.x)];
    const uint32_t all = b.bb.tile_count[it.x];
    const uint32_t thr = b.bb.slice_offset[b.total_tiles + 1], slice = b.bb.slice_offset[b.total_tiles + 2];
    const bool split = all > thr;
    const uint32_t first = split ? it.y * slice : 0u;
    const uint32_t cnt = split ? min(slice, all - first) : all;
    return raster_tile<TW, TH>(S, f.g, f.fb, (int)(it.x - f.tile_off), cnt,
                               b.bb.entries + b.bb.tile_offset[it.x] + first, b.depth_cull, phase, split);
}

// Raster over every frame's tiles in one launch.  Persistent form (the default): a grid of
// SMs x resident CTAs, each CTA taking the next item of the device-side (frame, tile)
// queue -- the item list, split tiles' slices first -- from a counter (b.queue, zeroed by
// batch_items_kernel) until the queue is empty.  The item is claimed by thread 0 and read
// by every thread after a barrier, so the whole CTA leaves the loop together.  The other
// form launches one CTA per item and leaves the balancing to the hardware block scheduler.
template <int TW, int TH, bool kPersistent>
__global__ void __launch_bounds__(kRasterThreads, kRasterMinBlocks) batch_raster_kernel(BatchDev b)
{
    __shared__ TileSmem<TW, TH> S;
    __shared__ uint32_t s_item;
    if (b.bb.tile_offset[b.total_tiles] > b.bb.capacity) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *b.overflow = 1;
        return;
    }
    const uint32_t nitems = min(b.bb.slice_offset[b.total_tiles], b.bb.item_capacity);
    if (!kPersistent && blockIdx.x >= nitems) return;
    uint32_t phase = 0;
    if (!kPersistent) {
        batch_raster_item<TW, TH>(S, b, blockIdx.x, phase);
        return;
    }
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(b.queue, 1u);
        block_sync();
        const uint32_t i = s_item;   // thread 0 writes the next claim only after raster_tile's last barrier
        if (i >= nitems) break;
        if (!batch_raster_item<TW, TH>(S, b, i, phase)) break;
    }
}

// blocks[i] = (frame, first cell): runs of kBatchRun frame cells per lane (resolve_run),
// written with one store per buffer when the frame's outputs are aligned.  Four resident
// blocks per SM (64 registers, no spills): the winners' record loads are latency-bound, and
// the fourth block's loads in flight took config 3 from 3.33 to 3.22 ms.
constexpr int kBatchRun = 2;
static_assert(kBatchResolveChunk % (kBatchRun * 256) == 0, "whole runs, the same trip count in every warp");

__global__ void __launch_bounds__(256, 4) batch_resolve_kernel(BatchDev b, const int2 *__restrict__ blocks)
{
    // the frame's descriptor in shared memory: read there, its fields are not reloaded
    // from global memory after each of the block's output stores
    __shared__ BatchFrame sf;
    const int2 blk = blocks[blockIdx.x];
    if (threadIdx.x == 0) sf = b.frames[blk.x];
    block_sync();
    const BatchFrame &f = sf;
    const uint64_t nz = (uint64_t)f.g.w * f.g.h;
    const uint64_t ncells = f.g.image ? nz + f.g.h : nz;
    const uint64_t end = min(ncells, (uint64_t)blk.y + kBatchResolveChunk);   // chunks start on runs
    if (!(f.g.w & 1)) {
        // an even-width frame by pairs of cells (resolve_even), four per thread at a time
        const uint64_t pend = (end + 1) / 2;
        for (uint64_t p0 = (uint64_t)blk.y / 2; p0 < pend; p0 += 4 * blockDim.x)
            resolve_even<4>(f.g, f.fb, p0 + threadIdx.x, blockDim.x, pend, f.vec != 0);
        return;
    }
    const int lane = threadIdx.x & 31;
    for (uint32_t i = threadIdx.x; i < kBatchResolveChunk / kBatchRun; i += blockDim.x) {
        const uint64_t p = (uint64_t)blk.y / kBatchRun + i;
        resolve_run<kBatchRun>(f.g, f.fb, p, kBatchRun * p < end, lane, f.vec != 0);
    }
}

cudaError_t prepare_batch_kernels()
{
    const int bytes = (int)setup_smem_bytes(kMaxTrianglesPerBlock, true);
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(batch_setup_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) ||
        (e = cudaFuncSetAttribute(batch_setup_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    return cudaFuncSetAttribute(batch_newline_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                128 * 1024);
}

cudaError_t launch_batch_vertex(const BatchDev &b, const int2 *blocks, uint32_t nblocks, cudaStream_t s)
{
    if (!nblocks) return cudaSuccess;
    batch_vertex_kernel<<<nblocks, 256, 0, s>>>(b, blocks);
    return cudaGetLastError();
}

cudaError_t launch_batch_setup(const BatchDev &b, const int2 *blocks, uint32_t nblocks, cudaStream_t s)
{
    if (!nblocks) return cudaSuccess;
    if (!valid_triangles_per_block(b.tpb)) return cudaErrorInvalidValue;
    const size_t smem = setup_smem_bytes(b.tpb, b.direct_max > 0);   // prepare_batch_kernels: above 48 KB
    const dim3 grid(nblocks), block(setup_block_threads(b.tpb));
    const bool chunks = b.tpb > kSetupChunk;
    if (b.direct_max > 0) {
        if (chunks) batch_setup_kernel<true, true><<<grid, block, smem, s>>>(b, blocks);
        else batch_setup_kernel<true, false><<<grid, block, smem, s>>>(b, blocks);
    } else {
        if (chunks) batch_setup_kernel<false, true><<<grid, block, smem, s>>>(b, blocks);
        else batch_setup_kernel<false, false><<<grid, block, smem, s>>>(b, blocks);
    }
    return cudaGetLastError();
}

cudaError_t launch_batch_newline(const BatchDev &b, const int2 *blocks, uint32_t nblocks, int max_nl,
                                 cudaStream_t s)
{
    if (!nblocks) return cudaSuccess;
    const size_t smem = 2 * (size_t)max_nl * sizeof(int32_t);
    if (smem <= 128 * 1024) batch_newline_kernel<true><<<nblocks, 1024, smem, s>>>(b, blocks);
    else batch_newline_kernel<false><<<nblocks, 1024, 0, s>>>(b, blocks);
    return cudaGetLastError();
}

cudaError_t launch_batch_bin_large(const BatchDev &b, bool fill, cudaStream_t s)
{
    const int grid = 8 * device_sm_count();   // eight CTAs of 8 warps per SM; the warps stride over the items
    if (fill) batch_bin_large_kernel<true><<<grid, 256, 0, s>>>(b);
    else batch_bin_large_kernel<false><<<grid, 256, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_batch_fill(const BatchDev &b, cudaStream_t s)
{
    batch_fill_kernel<<<kFillMinBlocks * 2 * device_sm_count(), kSetupThreads, 0, s>>>(b);
    return cudaGetLastError();
}

// Resident CTAs per SM of a raster kernel (looked up once per kernel and device).
template <class K>
static int resident_ctas(K kernel)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kRasterThreads, 0) != cudaSuccess || n < 1) n = 1;
    return n;
}

cudaError_t launch_batch_raster(const BatchDev &b, int tw, int th, bool persistent, cudaStream_t s)
{
    if (!b.total_tiles) return cudaSuccess;
    // persistent: SMs x resident CTAs take items from the queue; otherwise one CTA per
    // possible raster item, CTAs past the item count exiting at once
#define SLOTH_BATCH_RASTER_CASE(W_, H_)                                                        \
    if (tw == W_ && th == H_) {                                                                \
        if (persistent) {                                                                      \
            static int per_sm[64];                                                             \
            int dev = 0;                                                                       \
            cudaGetDevice(&dev);                                                               \
            if (dev >= 0 && dev < 64 && !per_sm[dev]) per_sm[dev] = resident_ctas(batch_raster_kernel<W_, H_, true>); \
            const uint32_t slots = (uint32_t)device_sm_count() * (dev >= 0 && dev < 64 ? per_sm[dev] : 1); \
            const uint32_t grid = slots < b.bb.item_capacity ? slots : b.bb.item_capacity;     \
            batch_raster_kernel<W_, H_, true><<<grid, kRasterThreads, 0, s>>>(b);              \
        } else {                                                                               \
            batch_raster_kernel<W_, H_, false><<<b.bb.item_capacity, kRasterThreads, 0, s>>>(b); \
        }                                                                                      \
        return cudaGetLastError();                                                             \
    }
    SLOTH_TILE_SHAPES(SLOTH_BATCH_RASTER_CASE)
#undef SLOTH_BATCH_RASTER_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_batch_items(const BatchDev &b, cudaStream_t s)
{
    if (!b.total_tiles) return cudaSuccess;
    batch_items_kernel<<<(b.total_tiles + 255) / 256, 256, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_batch_resolve(const BatchDev &b, const int2 *blocks, uint32_t nblocks, cudaStream_t s)
{
    if (!nblocks) return cudaSuccess;
    batch_resolve_kernel<<<nblocks, 256, 0, s>>>(b, blocks);
    return cudaGetLastError();
}

}  // namespace sloth
