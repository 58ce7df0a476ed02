// sloth_kernels.h -- host-visible launch interface of the GB300 kernels.
//
// The C ABI (sloth_api.cpp) owns device memory and calls these launchers on the
// context's stream.  Each launcher enqueues one kernel and returns the launch status.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sloth {

struct TriRecord;

// Geometry of one frame's target-cell tiling (mirrors Viewport in sloth_internal.cuh).
struct FrameGeom {
    int32_t w, h, image;
    int32_t tw, th, ntx, nty, pitch;
    int32_t nl_size;         // power of two >= h: leaves of the newline segment tree
    int32_t direct_max;      // triangles whose sample range holds 1..direct_max samples are
                             // rasterized by the setup kernel straight into the global keys
                             // (direct.cuh) instead of being binned; 0: none.  Needs every
                             // tile's keys valid for the current generation before setup.
};

// Device buffers of one frame (one Context).
struct FrameBuffers {
    uint64_t *keys;          // nty*th rows x pitch cells, valid where tile_gen == gen
    uint32_t *tile_gen;      // ntx*nty
    int32_t *nltree;         // 2*nl_size: max segment tree over rows of the draw indices whose
                             // newline row range [y0,y1) covers each node (-1 = none)
    TriRecord *records;      // draw index -> record
    uint32_t *rows;          // draw index -> sample rows y0 | y1 << 16 (setup writes, the newline reads)
    float *z_out;            // w*h
    uint32_t *cells_out;     // w*h (+h)
    int32_t *winner_out;     // w*h
    unsigned long long *fragments;   // covered-sample counter
    uint32_t *error;         // nonzero once a kernel gave up waiting for its copies (until the next clear)
    uint32_t gen;            // current clear generation (never 0)
    uint32_t wait_test;      // test hook: tile loads wait for 16 bytes that never come, briefly
};

// Binning scratch of one draw.
struct BinBuffers {
    uint32_t *tile_count;    // ntiles: before the scan the entries of small triangles whose
                             // first tile it is (each with its slot from the count), after it
                             // all the tile's entries
    uint32_t *tile_offset;   // ntiles + 1 (exclusive scan; [ntiles] = total entries)
    uint32_t *tile_cursor;   // ntiles: before the scan the tile's other entries (counted without
                             // a slot), after it the next of their slots
    uint64_t *entries;       // capacity: per tile, (ordered depth lower bound << 32 | draw index)
    uint32_t capacity;
    uint32_t *large_queue;   // large_cap mesh-local indices of triangles binned by warps: big
                             // ones from the front, the others from the back (bin_common.cuh)
    uint32_t *large_count;   // 3: big triangles queued, other large triangles queued, and
                             // (contexts) small binned triangles listed in fill_list
    uint32_t large_cap;
    uint2 *fill_list;        // large_cap: (draw-local index, slot in its first tile) of the
                             // small binned triangles (setup appends, the fill walks them);
                             // null: none kept
    uint32_t *slice_offset;  // ntiles + kSliceExtra: per tile the first raster item of its
                             // slices within its class (item_offset); [ntiles] = items,
                             // [ntiles+1] = split threshold, [ntiles+2] = slice size,
                             // [ntiles+3] = items of split tiles (listed first), [ntiles+4] =
                             // first item of the light tiles (listed last), [ntiles+5] = the
                             // light threshold (entries)
    uint2 *items;            // item_capacity: (tile, slice) of each raster CTA
    uint32_t item_capacity;
    uint32_t *max_total;     // optional: the scan folds each draw's entry total in (atomicMax)
};

// A tile holding many more entries than the launch's mean is rasterized in slices by
// separate CTAs, which fold their keys into the tile's with a 64-bit global atomicMin (the
// minimum is order-independent, so the result is the same), and its slices are listed
// before every other item so that they start first.  Without it a very dense small
// viewport (hundreds of thousands of triangles over a few tiles) leaves a few CTAs working
// long after the rest of the GPU is idle.  Split threshold: the smaller of 4 x the mean
// entries of a non-empty tile and 2 x total / kTargetItems (so that a launch of few, evenly
// heavy tiles still spreads over the GPU), at least kMinSplitEntries; slices hold half the
// threshold.
constexpr uint32_t kMinSplitEntries = 2048;
constexpr uint32_t kTargetItems = 1024;

struct SplitParams {
    uint32_t threshold, slice;
};

__host__ __device__ inline uint32_t tile_slices(uint32_t n, SplitParams sp)
{
    return n == 0 ? 0u : (n <= sp.threshold ? 1u : (n + sp.slice - 1) / sp.slice);
}

constexpr uint32_t kSliceExtra = 6;   // entries of slice_offset past the tiles

// The first raster item of tile t (cnt entries) among the three classes the scan numbers:
// split tiles' slices, then the other tiles, then the light ones.
__host__ __device__ inline uint32_t item_offset(const uint32_t *so, uint32_t ntiles, uint32_t t, uint32_t cnt,
                                               uint32_t split_threshold)
{
    const uint32_t base = cnt > split_threshold ? 0u : (cnt < so[ntiles + 5] ? so[ntiles + 4] : so[ntiles + 3]);
    return so[t] + base;
}

// Raster CTAs needed for ntiles tiles holding at most `capacity` entries in total.
inline uint32_t raster_item_bound(uint32_t ntiles, size_t capacity)
{
    return (uint32_t)(ntiles + capacity / (kMinSplitEntries / 2) + 1);
}

// A mesh on the device.  Setup takes an indexed mesh's triangles in a spatial order
// (order[p]: the triangle at position p; oidx: its three vertex indices, at 3p) so that the
// triangles of one warp or block lie close together on screen; every output stays indexed
// by the triangle itself, and the results do not depend on the order.  order and oidx are
// nullptr for the mesh's own order.
struct MeshDev {
    const float *x, *y, *z;  // nvert
    const uint32_t *idx;     // 3*ntri or nullptr (soup)
    const uint8_t *rgb;      // 3*ntri
    uint32_t nvert, ntri;
    const uint32_t *order = nullptr;   // ntri or nullptr
    const uint32_t *oidx = nullptr;    // 3*ntri or nullptr
};

struct Mat4 {
    float m[16];             // row-major
};

// Triangles per block of the setup kernels: a tuning choice, the results do not depend on
// it.  A block has min(tpb, kSetupThreads) threads, and each thread takes tpb / threads
// triangles in turn (consecutive threads, consecutive triangles), so that a triangle's
// record stores and key reductions drain while the thread sets up the next.  The fills walk
// the list setup made, a grid of kFillMinBlocks * 2 blocks per SM.
constexpr int kSetupThreads = 256;
constexpr int kSetupMinBlocks = 3;   // resident setup blocks per SM the register budget keeps (direct path)
constexpr int kFillMinBlocks = 4;    // the same for the fill kernels and setup without the direct path
constexpr int kDefaultTrianglesPerBlock = 256;
constexpr int kTrianglesPerBlockChoices[4] = {128, 256, 1024, 4096};
constexpr int kMaxTrianglesPerBlock = 4096;
inline bool valid_triangles_per_block(long long v) { return v == 128 || v == 256 || v == 1024 || v == 4096; }
__host__ __device__ inline int setup_block_threads(int tpb) { return tpb < kSetupThreads ? tpb : kSetupThreads; }
// A setup block takes its triangles in chunks of at most kSetupChunk.  Phase 1 of a chunk
// queues, in shared memory, the triangles that need the rest of their setup together with
// their transformed vertices and colour (record.cuh: SetupStash, 44 bytes a triangle).
constexpr int kSetupChunk = 1024;
__host__ __device__ inline int setup_chunk(int tpb) { return tpb < kSetupChunk ? tpb : kSetupChunk; }
// Dynamic shared memory of a setup block: the stash, and with the direct path one stage of
// 23 x 32 words per warp (direct.cuh) after it.
__host__ __device__ inline size_t setup_smem_bytes(int tpb, bool direct = false)
{
    return 44u * (size_t)setup_chunk(tpb) + (direct ? (size_t)(setup_block_threads(tpb) / 32) * 23u * 32u * 4u : 0u);
}
// Sets the shared-memory limit of the setup kernels with the direct path (above the 48 KB
// default), once per device; call before the first launch and outside stream capture.
cudaError_t prepare_setup_kernels();

// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount, looked
// up once per device): grids of the grid-stride kernels are sized by it.
int device_sm_count();

// frame resets (error word, fragments, newline tree) and draw resets (tile counts, large
// queue counters), either or both, in one launch; tiles_current also sets every tile's
// generation to the current one (its keys were cleared to the empty key before).
// Every key a sample can write in ncells cells of tile rows of tw cells (a multiple of tw)
// set to the empty key: the even half of each tile row when the frame's width is even
// (key_col), all of them otherwise.
cudaError_t launch_clear_keys(uint64_t *keys, uint64_t ncells, int tw, bool even_width, cudaStream_t s);
cudaError_t launch_frame_reset(const FrameBuffers &fb, const BinBuffers &bb, uint32_t nl_nodes, uint32_t ntiles,
                               bool frame, bool draw, bool tiles_current, cudaStream_t s);

// vertex transform: tv[i] = (M*v_i).xyz (nalgebra order), float4 per vertex.
cudaError_t launch_vertex_transform(const MeshDev &mesh, const Mat4 &M, float4 *tv,
                                    cudaStream_t s);

// per-triangle setup: records[tri_base + t], small-triangle tile counts and newline rows,
// large-triangle queue.  tv: the vertex kernel's output, or null to transform by M here
// (soups only: mesh.idx null).
cudaError_t launch_setup(const MeshDev &mesh, const float4 *tv, const Mat4 &M, uint32_t tri_base,
                         const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                         cudaStream_t s, int tpb = kDefaultTrianglesPerBlock);
// newline sentinels (image mode): fold each triangle's row range into the segment tree.
// The packed rows are in setup's order of the mesh: order is the mesh's MeshDev::order.
cudaError_t launch_newline(uint32_t ntri, const uint32_t *order, uint32_t tri_base, const FrameGeom &g,
                           const FrameBuffers &fb, cudaStream_t s);
cudaError_t launch_bin_count_large(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                                   const BinBuffers &bb, cudaStream_t s);
cudaError_t launch_bin_scan(uint32_t ntiles, const BinBuffers &bb, cudaStream_t s);
cudaError_t launch_bin_items(uint32_t ntiles, const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                             cudaStream_t s);
// small binned triangles' tile entries: the ones setup listed in bb.fill_list
cudaError_t launch_bin_fill(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                            cudaStream_t s);
cudaError_t launch_bin_fill_large(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                                  const BinBuffers &bb, cudaStream_t s);

// per-tile raster: 64-bit atomicMin of depth keys in shared memory, merged into keys.  A
// draw whose tile entries outgrew the entry buffer (the scan total is above the capacity;
// its fill wrote what fitted) is rasterized by the same launch without tiles: the item
// kernel has made every tile's keys current, and one warp per binned triangle of the draw
// (ntri triangles from tri_base) folds its covered samples straight into the global keys.
cudaError_t launch_raster(const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb, int depth_cull,
                          uint32_t ntri, uint32_t tri_base, cudaStream_t s);

// resolve: keys -> z, frame cells, winners.
cudaError_t launch_resolve(const FrameGeom &g, const FrameBuffers &fb, cudaStream_t s);

constexpr int kTileW = 64;   // default tile: cells (even)
constexpr int kTileH = 32;   // rows

// Tile shapes the raster is compiled for, (cells, rows); the autotuner picks among them.
#define SLOTH_TILE_SHAPES(X) X(64, 32) X(32, 16) X(64, 16) X(32, 32) X(128, 16)
constexpr int kNumTileShapes = 5;
constexpr int kTileShapes[kNumTileShapes][2] = {{64, 32}, {32, 16}, {64, 16}, {32, 32}, {128, 16}};
constexpr uint32_t kSmallMaxTiles = 8;   // triangles over more tiles are binned by warps

}  // namespace sloth
