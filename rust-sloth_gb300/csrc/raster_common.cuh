// raster_common.cuh -- the per-tile raster shared by the single-frame and batched kernels.
//
// Replaces the sample loop of src/rasterizer.rs:69-86.  One CTA owns one tile of depth
// cells (TH rows x TW cells).  Its warps take the tile's triangle entries one at a time;
// the 32 lanes walk the triangle's samples inside the tile (unwrapped and wrapped parts),
// evaluate the three edge functions and the barycentric depth in the reference's f32
// operation order, and fold (depth, draw index) keys into the tile with a 64-bit
// shared-memory atomicMin.  The minimum key of a cell is the reference's last successful
// depth write.  Keys of earlier draws since the clear are merged in first.
//
// Depth culling (on by default): entries carry a proven lower bound of every depth their
// triangle can produce in this tile (bounds.cuh).  The CTA orders its entries front to
// back by a counting sort into depth buckets (one pass of shared atomics, not a sorting
// network) and keeps an upper bound of the farthest key depth among the tile's writable
// cells.  An entry whose bound is strictly above it cannot win any cell; when the
// smallest bound of the bucket a window of entries starts in is above it, neither can
// any entry left, so the warps stop there.  Only skipped work changes: the buffers are
// the same bit for bit; the fragment counter then counts only the fragments of the
// triangles that were rasterized.
#pragma once

#include "sloth_internal.cuh"
#include "sloth_kernels.h"

namespace sloth {

constexpr int kSortCap = 2048;   // entries ordered per pass (16 KB of shared memory)
constexpr int kDepthBuckets = 256;   // depth buckets of the counting sort (= kRasterThreads)
constexpr int kRasterThreads = 256;
static_assert(kDepthBuckets == kRasterThreads, "one bucket per thread in the scan");
constexpr int kRasterMinBlocks = 5;   // resident CTAs per SM the register budget allows

template <int TW, int TH>
struct TileSmem {
    alignas(128) unsigned long long keys[TH * TW];   // bulk-copy target: 16-byte aligned rows
    unsigned long long kbar;                          // mbarrier of the tile load
    uint32_t kok;                                     // the tile load arrived
    unsigned long long ent[kSortCap];
    uint32_t bcount[kDepthBuckets];     // entries per depth bucket, then the scatter cursors
    uint32_t bstart[kDepthBuckets + 1]; // first entry of each bucket (exclusive scan)
    uint32_t bmin[kDepthBuckets];       // smallest depth bound in each bucket
    uint32_t zlo_min, zlo_max;
    uint32_t next, zmax_u, zmax_w;
    uint32_t rmu[32], rmw[32];          // the same bounds per row of the tile
    uint32_t frags[kRasterThreads / 32];
};

// ---- bulk copies of the key tile (cp.async.bulk, completion on an mbarrier) ----

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Waits at most `limit` polls for phase `parity` of the barrier; false when it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity, uint32_t limit)
{
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void bulk_load(void *sdst, const void *gsrc, uint32_t bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sdst)),
                 "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void bulk_store(void *gdst, const void *ssrc, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_u32(ssrc)),
                 "r"(bytes)
                 : "memory");
}

// Waits until every bulk store of the thread has read its shared-memory source, so that
// the block may leave; the global writes complete by the end of the grid, before any
// later kernel reads the keys (nothing in this grid reads a tile another block stores).
__device__ __forceinline__ void bulk_store_drain()
{
    asm volatile("cp.async.bulk.commit_group;\ncp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Orders this thread's generic-proxy shared-memory writes before later async-proxy
// (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

constexpr uint32_t kWaitPolls = 1u << 22;   // polls of a bulk-copy barrier before giving up
constexpr uint32_t kTestWaitPolls = 1u << 10;   // the same under the wait test hook

// One sample of the reference's loop body: edge test, depth, key folded into the tile.
// With a depth bound zb of the triangle in this tile (0: none), a cell already nearer
// than zb is passed over before the edge test: no depth of the triangle can beat it.
template <int TW, int kNotWrapped>
__device__ __forceinline__ void fold_sample(const TriRecord &r, uint32_t gtri, int x, int y, int R0, int C0,
                                            int w, unsigned long long *skeys, uint32_t &frags, uint32_t zb,
                                            const EdgeRows *rows = nullptr)
{
    const int row = kNotWrapped ? (y - R0) : (y + 1 - R0);
    const int col = kNotWrapped ? (2 * x - C0) : (2 * x - w - C0);
    unsigned long long *p = &skeys[row * TW + key_col(col, TW)];
    if (zb > *(volatile const uint32_t *)(reinterpret_cast<const uint32_t *>(p) + 1)) return;
    // with the row's edge terms given (a walk along one row), only the column terms remain
    const EdgeVals e = rows ? eval_edges_row(r, *rows, (float)x) : eval_edges(r, (float)x, (float)y);
    if (e.w0 >= 0.0f && e.w1 >= 0.0f && e.w2 >= 0.0f) {
        ++frags;
        const float z = interp_z(r.v1z, r.dz2, r.dz3, r.a, e.w1, e.w2);
        if (z < kFltMax) {
            const unsigned long long key = make_key(z, gtri, kNotWrapped);
            if (key < *(volatile unsigned long long *)p) atomicMin(p, key);
        }
    }
}

// One edge's columns on one row: for records with kFlagFiniteXY the edge value
// w(x) = fl(A - fl(dy * fl(x - ax))), A = fl(dx * fl(py - ay)), is monotone in x (a chain of
// correctly rounded monotone operations, no overflow), so the columns where w >= 0 are a
// prefix (dy > 0), a suffix (dy < 0) or all or none (dy == 0) of the row.  The real-valued
// crossing only estimates the end; the exact value at the first column past it decides
// (stepping on while it still passes), so [lo, hi) keeps every column that passes.
__device__ __forceinline__ void edge_row_span(float dx, float dy, float ax, float ay, float py, int &lo, int &hi)
{
    if (lo >= hi) return;
    if (dy == 0.0f) {
        if (!(edge_eval(dx, dy, ax, ay, (float)lo, py) >= 0.0f)) hi = lo;
        return;
    }
    const float cross = ax + __fdividef(fmul(dx, fsub(py, ay)), dy);   // estimate only
    if (dy > 0.0f) {
        int t = (int)fminf(fmaxf(floorf(cross), (float)(lo - 1)), (float)(hi - 1)) + 1;
        while (t < hi && edge_eval(dx, dy, ax, ay, (float)t, py) >= 0.0f) ++t;
        hi = t;
    } else {
        int t = (int)fminf(fmaxf(ceilf(cross), (float)lo), (float)hi) - 1;
        while (t >= lo && edge_eval(dx, dy, ax, ay, (float)t, py) >= 0.0f) --t;
        lo = t + 1;
    }
}

// Parts of more samples than this are walked over their rows' column spans; smaller ones
// over the whole rectangle.
constexpr int kSpanMinSamples = 128;

// Walk the samples of rect c and fold covered samples' keys.  Large parts of records with
// kFlagFiniteXY: lane i bounds row c.ya + i to the columns that can pass all three edges
// (at most 32 rows: a part lies in one tile) -- none when the row's depth bound (rowmax,
// indexed by tile row) is below the entry's depth bound zb -- and the warp walks the
// concatenated spans
// 32 samples at a time, each lane finding its row by a binary search over the spans'
// running ends.  Otherwise the rectangle, row-major, 32 samples at a time.  Every walked
// sample gets the exact test.
template <int TW, int kNotWrapped>
__device__ __forceinline__ void raster_part(const TriRecord &r, uint32_t gtri, Rect c, int R0,
                                            int C0, int w, unsigned long long *skeys, int lane,
                                            uint32_t &frags, const uint32_t *rowmax, uint32_t zb)
{
    if (c.empty()) return;
    const bool finite = (r.flags & kFlagFiniteXY) != 0;
    if (finite && !rect_may_cover(r, c)) return;
    const int bw = c.xb - c.xa;
    const int area = bw * (c.yb - c.ya);
    if (finite && area > kSpanMinSamples) {
        const int y = c.ya + lane;
        int lo = c.xa, hi = y < c.yb ? c.xb : c.xa;
        // a row whose every writable cell is nearer than the entry's depth bound is done
        if (hi > lo && zb > *(volatile const uint32_t *)&rowmax[kNotWrapped ? y - R0 : y + 1 - R0]) hi = lo;
        const float py = (float)y;
        edge_row_span(r.dx0, r.dy0, r.v2x, r.v2y, py, lo, hi);
        edge_row_span(r.dx1, r.dy1, r.v3x, r.v3y, py, lo, hi);
        edge_row_span(r.dx2, r.dy2, r.v1x, r.v1y, py, lo, hi);
        const int len = max(hi - lo, 0);
        int end = len;   // running end of the spans up to this row
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, end, d);
            if (lane >= d) end += o;
        }
        const int total = __shfl_sync(0xffffffffu, end, 31);
        const int xoff = lo - (end - len);   // column of span sample k of this row: k + xoff
        for (int base = 0; base < total; base += 32) {
            const int k = base + lane;
            // the row of sample k: the number of rows whose spans end at or before k
            int row = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xffffffffu, end, row + step - 1) <= k) row += step;
            const int x = k + __shfl_sync(0xffffffffu, xoff, row);
            if (k < total) fold_sample<TW, kNotWrapped>(r, gtri, x, c.ya + row, R0, C0, w, skeys, frags, zb);
        }
        return;
    }
    // floor(n / bw) for n <= 32 from a reciprocal: (n + 0.5) / bw is at least 0.5 / bw
    // from an integer, far beyond the reciprocal's rounding error
    const float rbw = __frcp_rn((float)bw);
    const int q = (int)(32.5f * rbw), rem = 32 - q * bw;
    int dy = (int)(((float)lane + 0.5f) * rbw), dx = lane - dy * bw;
    for (int k = lane; k < area; k += 32) {
        fold_sample<TW, kNotWrapped>(r, gtri, c.xa + dx, c.ya + dy, R0, C0, w, skeys, frags, zb);
        dx += rem;
        dy += q;
        if (dx >= bw) {
            dx -= bw;
            ++dy;
        }
    }
}

// ---- lane mode: one lane per entry (tiles of few entries, mostly small triangles) ----

// The part of a record's samples (unwrapped or wrapped) that falls in tile (tr, tc),
// clipped to the tile; empty when the exact corner test shows no covered sample.
template <int kNotWrapped>
__device__ __forceinline__ Rect tile_part(const TriRecord &r, const Viewport &vp, int tr, int tc)
{
    const Rect p = kNotWrapped ? unwrapped_part(vp, r.x0, r.xe, r.y0, r.y1) : wrapped_part(vp, r.x0, r.xe, r.y0, r.y1);
    if (p.empty()) return Rect{0, 0, 0, 0};
    const Rect c = kNotWrapped ? clip_unwrapped(vp, p, tr, tc) : clip_wrapped(vp, p, tr, tc);
    if (c.empty() || ((r.flags & kFlagFiniteXY) && !rect_may_cover(r, c))) return Rect{0, 0, 0, 0};
    return c;
}

__device__ __forceinline__ int rect_area(const Rect &c)
{
    return c.empty() ? 0 : (c.xb - c.xa) * (c.yb - c.ya);
}

// One lane walks every sample of rect c, row by row (each row's edge terms once).
template <int TW, int kNotWrapped>
__device__ __forceinline__ void raster_serial(const TriRecord &r, uint32_t gtri, const Rect &c, int R0, int C0,
                                              int w, unsigned long long *skeys, uint32_t &frags, uint32_t zb)
{
    for (int y = c.ya; y < c.yb; ++y) {
        const EdgeRows rows = edge_rows(r, (float)y);
        for (int x = c.xa; x < c.xb; ++x)
            fold_sample<TW, kNotWrapped>(r, gtri, x, y, R0, C0, w, skeys, frags, zb, &rows);
    }
}

// Entries whose clipped rectangles hold at most this many samples are walked by their
// lane alone; larger ones by the whole warp.  When most of a warp's window is small
// (meshes of tiny triangles), the lanes also take entries of up to kSerialWideSamples,
// each lane busy with its own; otherwise a lane walking one alone would hold its warp's
// walks of the large ones back.
constexpr int kSerialMaxSamples = 4;
constexpr int kSerialWideSamples = 16;

// Depth bounds: zmax_u / zmax_w are upper bounds of the farthest depth (ordered high key
// word) among the tile's cells that unwrapped samples can write (row y in [1,h-2], column
// 2x in [2,w-1], even) and among those wrapped samples can write (row y+1 in [2,h-1],
// column 2x-w in [0,w-4], of the parity of w); rmu[i] / rmw[i] are the same over tile row
// i.  Lane i of the refreshing warp reads row i: 16-byte reads of two keys of the row's
// even half (columns 4j and 4j+2), and of its odd half (4j+1, 4j+3) when w is odd, rotated
// by lane so that the lanes of a read hit different banks; it folds its maxima in with
// atomicMin.  Reads race with the atomics of other warps; key values only decrease, so
// every bound read stays an upper bound of every later state.
__device__ __forceinline__ void ld_hi2(uint32_t addr, uint32_t &hi0, uint32_t &hi1)
{
    uint32_t lo0, lo1;
    asm volatile("ld.volatile.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(lo0), "=r"(hi0), "=r"(lo1), "=r"(hi1)
                 : "r"(addr));
}

template <int TW, int TH>
__device__ __forceinline__ void refresh_bounds(TileSmem<TW, TH> &S, int R0, int C0, const FrameGeom &g, int lane)
{
    constexpr int Q = TW / 4;   // 16-byte reads per half row
    static_assert((Q & (Q - 1)) == 0, "rotation by mask");
    const int wpar = g.w & 1;
    uint32_t mu = 0, mw = 0;
    if (lane < TH) {
        const uint32_t even = smem_u32(S.keys) + 8u * (uint32_t)(lane * TW), odd = even + 4u * (uint32_t)TW;
        if (R0 >= 2 && R0 + TH <= g.h - 1 && C0 >= 2 && C0 + TW <= g.w - 3) {
            // every cell of the tile is writable: unwrapped samples write the even columns,
            // wrapped ones the columns of w's parity (C0 is even)
#pragma unroll 8
            for (int k = 0; k < Q; ++k) {
                const uint32_t off = 16u * (uint32_t)((k + lane) & (Q - 1));
                uint32_t h0, h1;
                ld_hi2(even + off, h0, h1);
                mu = max(mu, max(h0, h1));
                if (wpar) {
                    ld_hi2(odd + off, h0, h1);
                    mw = max(mw, max(h0, h1));
                }
            }
            if (!wpar) mw = mu;
        } else {
            const int gr = R0 + lane;
            const bool ru = gr >= 1 && gr <= g.h - 2, rw = gr >= 2 && gr <= g.h - 1;
            for (int k = 0; k < Q; ++k) {
                const int j = (k + lane) & (Q - 1);
                const int gc = C0 + 4 * j;   // columns gc, gc + 2 (even); gc + 1, gc + 3 (odd)
                uint32_t h0, h1;
                ld_hi2(even + 16u * (uint32_t)j, h0, h1);
                if (ru && gc >= 2 && gc <= g.w - 1) mu = max(mu, h0);
                if (ru && gc + 2 >= 2 && gc + 2 <= g.w - 1) mu = max(mu, h1);
                if (rw) {
                    if (wpar) ld_hi2(odd + 16u * (uint32_t)j, h0, h1);
                    if (gc + wpar <= g.w - 4) mw = max(mw, h0);
                    if (gc + 2 + wpar <= g.w - 4) mw = max(mw, h1);
                }
            }
        }
        atomicMin(&S.rmu[lane], mu);
        atomicMin(&S.rmw[lane], mw);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        mu = max(mu, __shfl_xor_sync(0xffffffffu, mu, d));
        mw = max(mw, __shfl_xor_sync(0xffffffffu, mw, d));
    }
    if (lane == 0) {
        atomicMin(&S.zmax_u, mu);
        atomicMin(&S.zmax_w, mw);
    }
}

// Rasterize one tile of one frame: `cnt` entries at `entries`.  Called by all threads of
// the CTA; returns after the tile's keys are stored and its generation is set, true, or
// false when the load of an earlier draw's keys did not arrive (the tile is left as it
// is, the error word is set, and the CTA must take no further tile).  A slice of a split
// tile (split true) starts from empty keys and folds its keys into the tile's with a
// global atomicMin; the tile's keys and generation were prepared before the launch.
// `phase` carries the tile-load barrier's state across the tiles of one CTA (0 before the
// first): bit 1 once thread 0 has initialised the barrier (at the CTA's first load),
// bit 0 the parity of the phase the next load completes.
template <int TW, int TH>
__device__ __forceinline__ bool raster_tile(TileSmem<TW, TH> &S, const FrameGeom &g, const FrameBuffers &fb,
                                            int tile, uint32_t cnt, const uint64_t *__restrict__ entries,
                                            int depth_cull, uint32_t &phase, bool split = false)
{
    static_assert(TH <= 32, "a tile part has at most 32 rows: one lane per row in raster_part");
    const int tr = tile / g.ntx, tc = tile - (tile / g.ntx) * g.ntx;
    const int R0 = tr * TH, C0 = tc * TW;
    const bool merge = !split && fb.tile_gen[tile] == fb.gen;
    unsigned long long *gk = reinterpret_cast<unsigned long long *>(fb.keys) + (size_t)R0 * g.pitch + C0;
    const int live = live_keys_per_row(g.w, TW);   // keys of a tile row that samples can write
    if (merge) {
        // keys of earlier draws since the clear: one bulk copy per tile row (live*8 bytes,
        // 16-byte aligned at both ends), completing on an mbarrier
        if (threadIdx.x < 32) {
            // warp 0: lane 0 arms the barrier for this phase, then the lanes issue one row each
            if (threadIdx.x == 0) {
                if (!(phase & 2u)) {
                    mbar_init(&S.kbar, 1);
                    fence_proxy_async_smem();
                }
                mbar_expect_tx(&S.kbar, (uint32_t)(TH * live * sizeof(unsigned long long)) + (fb.wait_test ? 16u : 0u));
            }
            __syncwarp();
            for (int rr = threadIdx.x; rr < TH; rr += 32)
                bulk_load(&S.keys[rr * TW], gk + (size_t)rr * g.pitch, live * sizeof(unsigned long long), &S.kbar);
        }
        block_sync();
        if (threadIdx.x == 0) {
            const uint32_t polls = fb.wait_test ? kTestWaitPolls : kWaitPolls;
            S.kok = (mbar_wait(&S.kbar, phase & 1u, polls) || mbar_wait(&S.kbar, phase & 1u, polls)) ? 1u : 0u;
        }
        block_sync();
        phase = (phase ^ 1u) | 2u;
        if (!S.kok) {
            // the copy did not arrive: report it and leave the tile as it is
            if (threadIdx.x == 0 && fb.error) atomicOr(fb.error, 1u);
            return false;
        }
    } else {
        for (int i = threadIdx.x; i < TH * TW; i += blockDim.x)
            if ((i & (TW - 1)) < live) S.keys[i] = kEmptyKey;
    }
    if (threadIdx.x == 0) S.zmax_u = S.zmax_w = 0xffffffffu;
    if (threadIdx.x < 64) (threadIdx.x < 32 ? S.rmu : S.rmw)[threadIdx.x & 31] = 0xffffffffu;

    const int lane = threadIdx.x & 31;
    const Viewport vp{g.w, g.h, g.image, g.tw, g.th, g.ntx, g.nty, g.pitch};
    uint32_t frags = 0;
    const int wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < cnt; base += kSortCap) {
        const uint32_t n = min(cnt - base, (uint32_t)kSortCap);
        if (!depth_cull) {
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) S.ent[i] = entries[base + i];
        } else {
            // Counting sort into kDepthBuckets buckets of the entries' depth bounds (front
            // to back): a bucket function monotone in the bound, so that bucket b's
            // smallest bound (bmin) grows with b; the order inside a bucket is free.
            if (threadIdx.x == 0) {
                S.zlo_min = 0xffffffffu;
                S.zlo_max = 0u;
            }
            S.bcount[threadIdx.x] = 0u;
            S.bmin[threadIdx.x] = 0xffffffffu;
            block_sync();
            // range of the finite bounds (-inf bounds, of triangles without a usable
            // bound, go to bucket 0)
            uint32_t lmin = 0xffffffffu, lmax = 0u;
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                const uint32_t z = (uint32_t)(entries[base + i] >> 32);
                if (isfinite(float_of_ordered(z))) {
                    lmin = min(lmin, z);
                    lmax = max(lmax, z);
                }
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                lmin = min(lmin, __shfl_xor_sync(0xffffffffu, lmin, d));
                lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, d));
            }
            if (lane == 0) {
                atomicMin(&S.zlo_min, lmin);
                atomicMax(&S.zlo_max, lmax);
            }
            block_sync();
            // buckets linear in depth over [fmin, fmax]: monotone in the bound
            const bool any = S.zlo_min <= S.zlo_max;
            const float fmin = any ? float_of_ordered(S.zlo_min) : 0.0f;
            const float fspan = any ? float_of_ordered(S.zlo_max) - fmin : 0.0f;
            const float scale = fspan > 0.0f ? (float)kDepthBuckets / fspan : 0.0f;
            auto bucket = [&](uint32_t z) {
                const float f = float_of_ordered(z);
                if (!(f > fmin)) return 0u;
                const float q = (f - fmin) * scale;
                return q < (float)(kDepthBuckets - 1) ? (uint32_t)q : (uint32_t)kDepthBuckets - 1;
            };
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                const uint32_t z = (uint32_t)(entries[base + i] >> 32);
                const uint32_t b = bucket(z);
                atomicAdd(&S.bcount[b], 1u);
                atomicMin(&S.bmin[b], z);
            }
            block_sync();
            {
                // exclusive scan of the 256 counts, one per thread
                __shared__ uint32_t ws[kRasterThreads / 32];
                const uint32_t v = S.bcount[threadIdx.x];
                uint32_t x = v;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t o = __shfl_up_sync(0xffffffffu, x, d);
                    if (lane >= d) x += o;
                }
                if (lane == 31) ws[wid] = x;
                block_sync();
                uint32_t pre = x - v;
                for (int w = 0; w < wid; ++w) pre += ws[w];
                S.bstart[threadIdx.x] = pre;
                S.bcount[threadIdx.x] = pre;   // scatter cursor
                if (threadIdx.x == 0) S.bstart[kDepthBuckets] = n;
            }
            block_sync();
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                const unsigned long long e = entries[base + i];
                S.ent[atomicAdd(&S.bcount[bucket((uint32_t)(e >> 32))], 1u)] = e;
            }
        }
        if (threadIdx.x == 0) S.next = 0;
        block_sync();
        // Windows of kRasterThreads sorted entries, each in 8 interleaved slots: lane i of
        // slot j takes entry j + 8i, so that a warp's lanes spread over the window and the
        // warps move through the sorted order together.  The warps claim slots in order
        // from a shared counter, so that a warp done early takes more.  Each lane loads its
        // own record; a small triangle is walked by its lane, a larger one by the whole
        // warp (in the warp's sorted order, checked against the depth bound before each).
        constexpr uint32_t kSlots = kRasterThreads / 32;
        uint32_t wb = 0;          // warp-uniform: the bucket of the current window's first entry
        // warp-uniform count of warp walks since the warp's last refresh of the bound: one
        // refresh per 8 walks of a warp (culled entries do not count), warp w's first
        // after 1 + w walks
        uint32_t since = 7u - (uint32_t)wid;
        for (;;) {
            uint32_t claim = 0;
            if (lane == 0) claim = atomicAdd(&S.next, 1u);
            claim = __shfl_sync(0xffffffffu, claim, 0);
            const uint32_t w0 = (claim / kSlots) * kRasterThreads;
            if (w0 >= n) break;
            if (depth_cull) {
                // every entry from here on lies in bucket wb or later: when that bucket's
                // smallest bound is behind every writable cell, so is everything left
                while (S.bstart[wb + 1] <= w0) ++wb;
                // lane 0 decides for the warp: the bounds may fall between the lanes' reads,
                // and a warp that left the loop in part would wait on itself
                const uint32_t zu = *(volatile uint32_t *)&S.zmax_u, zw = *(volatile uint32_t *)&S.zmax_w;
                if (__shfl_sync(0xffffffffu, S.bmin[wb] > max(zu, zw) ? 1u : 0u, 0)) break;
            }
            const uint32_t e = w0 + claim % kSlots + kSlots * lane;
            const unsigned long long ent = e < n ? S.ent[e] : ~0ull;
            bool live = e < n;
            if (depth_cull && live) {
                const uint32_t zu = *(volatile uint32_t *)&S.zmax_u, zw = *(volatile uint32_t *)&S.zmax_w;
                if ((uint32_t)(ent >> 32) > (((uint32_t)ent & 0x80000000u) ? max(zu, zw) : zu)) live = false;
            }
            const uint32_t gtri = (uint32_t)ent & 0x7fffffffu;
            // the sample range (x0, xe, y0, y1) alone sizes the tile's part of the triangle
            int area = 0;
            if (live) {
                const int4 xr = __ldg(reinterpret_cast<const int4 *>(fb.records + gtri) + 4);
                const Rect U = unwrapped_part(vp, xr.x, xr.y, xr.z, xr.w);
                const Rect W = wrapped_part(vp, xr.x, xr.y, xr.z, xr.w);
                if (!U.empty()) area += rect_area(clip_unwrapped(vp, U, tr, tc));
                if (!W.empty()) area += rect_area(clip_wrapped(vp, W, tr, tc));
            }
            const int small = __popc(__ballot_sync(0xffffffffu, live && area <= kSerialWideSamples));
            const bool serial = live && area <= (small >= 16 ? kSerialWideSamples : kSerialMaxSamples);
            if (serial) {
                const TriRecord r = load_record(fb.records, gtri);
                const uint32_t zb = depth_cull ? (uint32_t)(ent >> 32) : 0u;
                raster_serial<TW, 1>(r, gtri, tile_part<1>(r, vp, tr, tc), R0, C0, g.w, S.keys, frags, zb);
                raster_serial<TW, 0>(r, gtri, tile_part<0>(r, vp, tr, tc), R0, C0, g.w, S.keys, frags, zb);
            }
            unsigned coop = __ballot_sync(0xffffffffu, live && !serial);
            while (coop) {
                if (depth_cull) {
                    if (since >= 8) {
                        refresh_bounds<TW, TH>(S, R0, C0, g, lane);
                        since = 0;
                    }
                    // every lane checks its own waiting entry against the bound; each
                    // decision stands on its own (the bound only falls), so the lanes may
                    // read different values
                    const uint32_t zu = *(volatile uint32_t *)&S.zmax_u, zw = *(volatile uint32_t *)&S.zmax_w;
                    const bool hidden = ((coop >> lane) & 1u) &&
                                        (uint32_t)(ent >> 32) > (((uint32_t)ent & 0x80000000u) ? max(zu, zw) : zu);
                    coop &= ~__ballot_sync(0xffffffffu, hidden);
                    if (!coop) break;
                    ++since;   // culled entries change no key: only walks count
                }
                const int src = __ffs(coop) - 1;
                coop &= coop - 1;
                const uint32_t gt = __shfl_sync(0xffffffffu, gtri, src);
                const uint32_t zb = depth_cull ? __shfl_sync(0xffffffffu, (uint32_t)(ent >> 32), src) : 0u;
                const TriRecord r = load_record(fb.records, gt);
                const Rect U = unwrapped_part(vp, r.x0, r.xe, r.y0, r.y1);
                if (!U.empty())
                    raster_part<TW, 1>(r, gt, clip_unwrapped(vp, U, tr, tc), R0, C0, g.w, S.keys, lane, frags,
                                       S.rmu, zb);
                const Rect W = wrapped_part(vp, r.x0, r.xe, r.y0, r.y1);
                if (!W.empty())
                    raster_part<TW, 0>(r, gt, clip_wrapped(vp, W, tr, tc), R0, C0, g.w, S.keys, lane, frags,
                                       S.rmw, zb);
            }
        }
        block_sync();
    }
    // fragment count: warp reduce, then one atomic per tile
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) frags += __shfl_xor_sync(0xffffffffu, frags, d);
    if (lane == 0) S.frags[threadIdx.x >> 5] = frags;
    __syncwarp();
    block_sync();
    if (!split) {
        // the tile's keys out: one bulk copy per row, issued once every thread's shared
        // writes are ordered before the async proxy
        fence_proxy_async_smem();
        block_sync();
        if (threadIdx.x < 32) {
            // warp 0: one row per lane, each lane waits for its own copies
            for (int rr = threadIdx.x; rr < TH; rr += 32)
                bulk_store(gk + (size_t)rr * g.pitch, &S.keys[rr * TW], live * sizeof(unsigned long long));
            bulk_store_drain();
        }
    } else {
        // shared and global keys share the layout: slot i of tile row rr is slot i globally
        for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
            const int rr = i / TW, cc = i - rr * TW;
            if (cc < live && S.keys[i] != kEmptyKey) red_min_u64(&gk[(size_t)rr * g.pitch + cc], S.keys[i]);
        }
    }
    if (threadIdx.x < 32) {
        // warp 0, converged: sum the per-warp counts, one atomic, tile generation
        uint32_t tot = lane < (int)(blockDim.x >> 5) ? S.frags[lane] : 0u;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, d);
        if (lane == 0) {
            atomicAdd(fb.fragments, (unsigned long long)tot);
            if (!split) fb.tile_gen[tile] = fb.gen;
        }
        __syncwarp();
    }
    block_sync();
    return true;
}

}  // namespace sloth
