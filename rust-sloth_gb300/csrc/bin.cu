// bin.cu -- binning of one frame's triangles into target-cell tiles.
//
// The reference visits every sample of every triangle's range in one sequential loop
// (src/rasterizer.rs:69-70).  Here each triangle is listed in the tiles whose depth
// cells it can write: count (setup kernel for small triangles, one warp per large
// triangle here), exclusive scan over tiles, then fill (bin_common.cuh).
#include "bin_common.cuh"
#include "direct.cuh"
#include "sloth_kernels.h"

namespace sloth {

__device__ __forceinline__ Viewport vp_of(const FrameGeom &g)
{
    return Viewport{g.w, g.h, g.image, g.tw, g.th, g.ntx, g.nty, g.pitch};
}

// Warps over the parts of the queued large triangles.
template <bool kFill>
__global__ void __launch_bounds__(256)
bin_large_kernel(uint32_t tri_base, FrameGeom g, FrameBuffers fb, BinBuffers bb)
{
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t items = large_items(bb.large_count);
    const Viewport vp = vp_of(g);
    for (uint32_t it = warp; it < items; it += nwarps) {
        uint32_t q, part, nparts;
        if (!large_item(it, bb.large_count, bb.large_cap, q, part, nparts)) break;
        const uint32_t gtri = tri_base + bb.large_queue[q];
        bin_large_warp<kFill>(fb.records + gtri, gtri, vp, bb.tile_count, bb.tile_cursor, bb.entries,
                              bb.capacity, lane, part, nparts);
    }
}

__device__ __forceinline__ SplitParams split_params(const BinBuffers &bb, uint32_t n)
{
    return SplitParams{bb.slice_offset[n + 1], bb.slice_offset[n + 2]};
}

// Exclusive scans of the tile entry counts (tile_count + tile_cursor: the entries with a
// counted slot and the others; offsets[n] = total) and of the raster items per tile, by one
// block, 4096 tiles per step with running carries.  Afterwards tile_count holds each tile's
// entries and tile_cursor the first slot after its counted ones.  A
// first pass sets the split threshold and the light threshold from the mean entries of a
// non-empty tile.  Items are numbered in three classes: split tiles' slices first (they
// start first), then the other tiles in tile order, then light tiles (fewer entries than
// a quarter of the mean: mostly the frame's nearly empty borders) last, so that the last
// wave of a launch is made of short CTAs.  slice_offset[t] is the tile's first item within
// its class; item_offset() adds the class base.
// The counted (tile_count) and other (tile_cursor) entries of tiles i0..i0+3, 0 past n;
// 16-byte loads when all four exist (i0 is a multiple of 4 and the arrays 16-byte aligned).
__device__ __forceinline__ void load_counts4(const BinBuffers &bb, uint32_t n, uint32_t i0, uint32_t c1[4],
                                             uint32_t c2[4])
{
    if (i0 + 4 <= n) {
        const uint4 a = *reinterpret_cast<const uint4 *>(bb.tile_count + i0);
        const uint4 b = *reinterpret_cast<const uint4 *>(bb.tile_cursor + i0);
        c1[0] = a.x; c1[1] = a.y; c1[2] = a.z; c1[3] = a.w;
        c2[0] = b.x; c2[1] = b.y; c2[2] = b.z; c2[3] = b.w;
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            c1[k] = i0 + k < n ? bb.tile_count[i0 + k] : 0u;
            c2[k] = i0 + k < n ? bb.tile_cursor[i0 + k] : 0u;
        }
    }
}

__global__ void __launch_bounds__(1024) bin_scan_kernel(uint32_t n, BinBuffers bb)
{
    constexpr int kV = 4;   // running sums: entries, split items, other items, light items
    __shared__ unsigned long long red_e[32];
    __shared__ uint32_t red_t[32];
    __shared__ uint32_t ws[kV][32];
    __shared__ uint32_t carry[kV];
    __shared__ SplitParams sp_s;
    __shared__ uint32_t light_s;
    const uint32_t tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    // pass 1: entries and non-empty tiles, four consecutive tiles per thread and step as in
    // pass 2; the first step's counts stay in registers for pass 2
    unsigned long long se = 0;
    uint32_t st = 0;
    uint32_t c1_0[4], c2_0[4];
    for (uint32_t base = 0; base < n; base += 4 * 1024) {
        uint32_t c1[4], c2[4];
        load_counts4(bb, n, base + 4 * tid, c1, c2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (base == 0) {
                c1_0[k] = c1[k];
                c2_0[k] = c2[k];
            }
            const uint32_t c = c1[k] + c2[k];   // counted and other entries
            se += c;
            st += c != 0u;
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        se += __shfl_xor_sync(0xffffffffu, se, d);
        st += __shfl_xor_sync(0xffffffffu, st, d);
    }
    if (lane == 0) {
        red_e[wid] = se;
        red_t[wid] = st;
    }
    if (tid < kV) carry[tid] = 0;
    block_sync();
    if (tid == 0) {
        unsigned long long te = 0;
        uint32_t tt = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            te += red_e[w];
            tt += red_t[w];
        }
        const unsigned long long mean = (te + (tt ? tt : 1u) - 1) / (tt ? tt : 1u);
        // 4x the mean, but low enough that a launch of few tiles still yields about
        // kTargetItems items to spread over the GPU
        unsigned long long thr = mean * 4 < 2 * te / kTargetItems ? mean * 4 : 2 * te / kTargetItems;
        if (thr < kMinSplitEntries) thr = kMinSplitEntries;
        sp_s.threshold = (uint32_t)(thr < 0x40000000ull ? thr : 0x40000000ull);
        sp_s.slice = sp_s.threshold / 2;
        light_s = (uint32_t)(mean / 4 < sp_s.threshold ? mean / 4 : sp_s.threshold);
    }
    block_sync();
    const SplitParams sp = sp_s;
    const uint32_t light = light_s;
    // pass 2: the scans
    for (uint32_t base = 0; base < n; base += 4 * 1024) {
        const uint32_t i0 = base + 4 * tid;
        uint32_t c[4], c1[4], c2[4], cls[4], loc[kV] = {0, 0, 0, 0};
        if (base == 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                c1[k] = c1_0[k];
                c2[k] = c2_0[k];
            }
        } else {
            load_counts4(bb, n, i0, c1, c2);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            c[k] = c1[k] + c2[k];
            cls[k] = c[k] > sp.threshold ? 1u : (c[k] < light ? 3u : 2u);
            loc[0] += c[k];
            loc[cls[k]] += tile_slices(c[k], sp);
        }
        uint32_t v[kV];
#pragma unroll
        for (int q = 0; q < kV; ++q) v[q] = loc[q];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
            for (int q = 0; q < kV; ++q) {
                const uint32_t o = __shfl_up_sync(0xffffffffu, v[q], d);
                if (lane >= d) v[q] += o;
            }
        }
        if (lane == 31)
#pragma unroll
            for (int q = 0; q < kV; ++q) ws[q][wid] = v[q];
        block_sync();
        if (wid == 0) {
            uint32_t a[kV];
#pragma unroll
            for (int q = 0; q < kV; ++q) a[q] = ws[q][lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
                for (int q = 0; q < kV; ++q) {
                    const uint32_t o = __shfl_up_sync(0xffffffffu, a[q], d);
                    if (lane >= d) a[q] += o;
                }
            }
#pragma unroll
            for (int q = 0; q < kV; ++q) ws[q][lane] = a[q];
        }
        block_sync();
        uint32_t p[kV];
#pragma unroll
        for (int q = 0; q < kV; ++q) p[q] = carry[q] + v[q] - loc[q] + (wid > 0 ? ws[q][wid - 1] : 0u);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (i0 + k < n) {
                // the first-tile entries take [offset, offset + c1) by their counted slots,
                // the others the slots after them from the cursor
                bb.tile_offset[i0 + k] = p[0];
                bb.tile_cursor[i0 + k] = p[0] + c1[k];
                bb.tile_count[i0 + k] = c[k];
                bb.slice_offset[i0 + k] = p[cls[k]];
            }
            p[0] += c[k];
            p[cls[k]] += tile_slices(c[k], sp);
        }
        block_sync();                    // every thread has read the carries
        if (tid == blockDim.x - 1)
#pragma unroll
            for (int q = 0; q < kV; ++q) carry[q] = p[q];
        block_sync();
    }
    if (tid == 0) {
        if (bb.max_total) atomicMax(bb.max_total, carry[0]);
        bb.tile_offset[n] = carry[0];
        bb.slice_offset[n] = carry[1] + carry[2] + carry[3];
        bb.slice_offset[n + 1] = sp.threshold;
        bb.slice_offset[n + 2] = sp.slice;
        bb.slice_offset[n + 3] = carry[1];
        bb.slice_offset[n + 4] = carry[1] + carry[2];
        bb.slice_offset[n + 5] = light;
    }
}

// One thread per tile: the raster items (tile, slice) of the tile, and for a tile that is
// rasterized in slices, its keys cleared (unless they hold keys of earlier draws since
// the clear) and its generation set before the slices fold into them.  When the draw's
// entries outgrew the buffer (the raster folds its triangles without tiles), every tile
// gets that treatment instead.
__global__ void __launch_bounds__(256)
bin_items_kernel(uint32_t n, FrameGeom g, FrameBuffers fb, BinBuffers bb)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (bb.tile_offset[n] > bb.capacity) {
        if (fb.tile_gen[t] != fb.gen) {
            const int tr = (int)t / g.ntx, tc = (int)t - tr * g.ntx;
            unsigned long long *k0 = reinterpret_cast<unsigned long long *>(fb.keys) +
                                     (size_t)tr * g.th * g.pitch + (size_t)tc * g.tw;
            for (int r = 0; r < g.th; ++r)
                for (int c = 0; c < live_keys_per_row(g.w, g.tw); ++c) k0[(size_t)r * g.pitch + c] = kEmptyKey;
            fb.tile_gen[t] = fb.gen;
        }
        return;
    }
    const SplitParams sp = split_params(bb, n);
    const uint32_t cnt = bb.tile_count[t], ns = tile_slices(cnt, sp);
    const bool split = cnt > sp.threshold;
    const uint32_t off = item_offset(bb.slice_offset, n, t, cnt, sp.threshold);
    for (uint32_t k = 0; k < ns && off + k < bb.item_capacity; ++k) bb.items[off + k] = make_uint2(t, k);
    if (split && fb.tile_gen[t] != fb.gen) {
        const int tr = (int)t / g.ntx, tc = (int)t - tr * g.ntx;
        unsigned long long *k0 = reinterpret_cast<unsigned long long *>(fb.keys) + (size_t)tr * g.th * g.pitch +
                                 (size_t)tc * g.tw;
        for (int r = 0; r < g.th; ++r)
            for (int c = 0; c < live_keys_per_row(g.w, g.tw); ++c) k0[(size_t)r * g.pitch + c] = kEmptyKey;
        fb.tile_gen[t] = fb.gen;
    }
}

// The small binned triangles setup listed, 256 per block and round (grid-stride): their
// tile entries.  Only their records are read.
__global__ void __launch_bounds__(kSetupThreads, kFillMinBlocks)
bin_fill_kernel(uint32_t tri_base, FrameGeom g, FrameBuffers fb, BinBuffers bb)
{
    const uint32_t n = bb.large_count[2];
    const Viewport vp = vp_of(g);
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool live = i < n;
        const uint2 e = live ? bb.fill_list[i] : make_uint2(0u, 0u);
        const uint32_t gtri = tri_base + e.x;
        TriRecord r;
        TileSpan sp{};
        if (live) {
            r = load_record(fb.records, gtri);
            sp = tile_span(vp, r);
        }
        fill_small_warp(live, r, gtri, vp, sp, bb.tile_offset, bb.tile_cursor, bb.entries, bb.capacity, e.y);
    }
}

static int large_grid()
{
    return 8 * device_sm_count();   // up to eight CTAs of 8 warps per SM; the warps stride over the items
}

cudaError_t launch_bin_count_large(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                                   const BinBuffers &bb, cudaStream_t s)
{
    bin_large_kernel<false><<<large_grid(), 256, 0, s>>>(tri_base, g, fb, bb);
    return cudaGetLastError();
}

cudaError_t launch_bin_scan(uint32_t ntiles, const BinBuffers &bb, cudaStream_t s)
{
    bin_scan_kernel<<<1, 1024, 0, s>>>(ntiles, bb);
    return cudaGetLastError();
}

cudaError_t launch_bin_items(uint32_t ntiles, const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                             cudaStream_t s)
{
    if (ntiles == 0) return cudaSuccess;
    bin_items_kernel<<<(ntiles + 255) / 256, 256, 0, s>>>(ntiles, g, fb, bb);
    return cudaGetLastError();
}

cudaError_t launch_bin_fill(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                            cudaStream_t s)
{
    bin_fill_kernel<<<kFillMinBlocks * 2 * device_sm_count(), kSetupThreads, 0, s>>>(tri_base, g, fb, bb);
    return cudaGetLastError();
}

cudaError_t launch_bin_fill_large(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                                  const BinBuffers &bb, cudaStream_t s)
{
    bin_large_kernel<true><<<large_grid(), 256, 0, s>>>(tri_base, g, fb, bb);
    return cudaGetLastError();
}

}  // namespace sloth
