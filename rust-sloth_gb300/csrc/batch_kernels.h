// batch_kernels.h -- device tables and launchers of the batched (many frames) path.
//
// A batch is a list of frames (viewport, image mode, utransform) and, per frame, an
// ordered list of draws (mesh, transform) -- the reference's per-frame loop over its
// mesh queue (src/main.rs:76-83) for many frames or views at once.  Every frame keeps its
// own depth keys, newline tree, records and outputs; draw indices inside a frame are
// frame-local, so every frame is bit-identical to drawing it alone.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "sloth_kernels.h"

namespace sloth {

struct BatchFrame {
    FrameGeom g;
    FrameBuffers fb;           // pointers into the batch's buffers, records offset to the frame
    uint32_t tile_off;         // first global tile of the frame
    uint32_t rec_off;          // first global record of the frame
    uint32_t first_draw;       // the frame's first draw
    uint32_t ndraws;
    uint64_t z_off;            // first depth cell of the frame in the batch's depth-cell order
    int32_t vec;               // the frame's outputs start on 8-byte boundaries: the resolve
                               // writes 2 cells per store
};

struct BatchDraw {
    MeshDev mesh;
    uint32_t frame;
    uint32_t rec_off;          // global record of the draw's first triangle
    uint32_t local_base;       // frame-local draw index of the draw's first triangle
    uint32_t vert_off;         // first transformed vertex of the draw
};

struct BatchDev {
    const BatchFrame *frames;
    const BatchDraw *draws;
    const Mat4 *mats;          // per draw: utransform * transform
    float4 *tv;                // transformed vertices of every draw
    uint32_t nframes, ndraws;
    uint32_t total_tiles;
    const uint32_t *frame_tile_off;   // nframes + 1 (for tile -> frame lookups)
    BinBuffers bb;             // global tile arrays and entries
    uint32_t *large_frame;     // frame of each large-queue entry
    uint32_t *overflow;        // set when the entries outgrew their capacity
    uint32_t *queue;           // the persistent raster's next item (zeroed by the item kernel)
    uint4 *fill_list;          // (frame, frame-local draw index, slot in its first tile, 0) of
                               // every small binned triangle, appended by setup: the fill walks
                               // only these
    uint32_t *fill_count;      // entries of fill_list (zeroed at the start of a render)
    int depth_cull;
    int tpb;                   // triangles per setup block (the triangle block table's step)
    int direct_max;            // the frames' FrameGeom::direct_max (the same for every frame)
};

// Block tables: one int2 (item, start) per block, built on the host.
cudaError_t launch_batch_vertex(const BatchDev &b, const int2 *blocks, uint32_t nblocks, cudaStream_t s);
cudaError_t launch_batch_setup(const BatchDev &b, const int2 *blocks, uint32_t nblocks, cudaStream_t s);
cudaError_t launch_batch_newline(const BatchDev &b, const int2 *blocks, uint32_t nblocks, int max_nl,
                                 cudaStream_t s);
cudaError_t launch_batch_bin_large(const BatchDev &b, bool fill, cudaStream_t s);
cudaError_t launch_batch_fill(const BatchDev &b, cudaStream_t s);
cudaError_t launch_batch_items(const BatchDev &b, cudaStream_t s);
cudaError_t launch_batch_raster(const BatchDev &b, int tw, int th, bool persistent, cudaStream_t s);
cudaError_t launch_batch_resolve(const BatchDev &b, const int2 *blocks, uint32_t nblocks, cudaStream_t s);
cudaError_t prepare_batch_kernels();

constexpr uint32_t kBatchNewlineChunk = 8192;   // triangles per newline block
constexpr uint32_t kBatchResolveChunk = 8192;   // cells per resolve block (four rounds of its threads)

}  // namespace sloth
