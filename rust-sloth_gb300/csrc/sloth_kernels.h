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
};

// Device buffers of one frame (one Context).
struct FrameBuffers {
    uint64_t *keys;          // nty*th rows x pitch cells, valid where tile_gen == gen
    uint32_t *tile_gen;      // ntx*nty
    int32_t *nltree;         // 2*nl_size: max segment tree over rows of the draw indices whose
                             // newline row range [y0,y1) covers each node (-1 = none)
    TriRecord *records;      // draw index -> record
    float *z_out;            // w*h
    uint32_t *cells_out;     // w*h (+h)
    int32_t *winner_out;     // w*h
    unsigned long long *fragments;   // covered-sample counter
    uint32_t gen;            // current clear generation (never 0)
};

// Binning scratch of one draw.
struct BinBuffers {
    uint32_t *tile_count;    // ntiles
    uint32_t *tile_offset;   // ntiles + 1 (exclusive scan; [ntiles] = total entries)
    uint32_t *tile_cursor;   // ntiles
    uint64_t *entries;       // capacity: per tile, (ordered depth lower bound << 32 | draw index)
    uint32_t capacity;
    uint32_t *large_queue;   // mesh-local triangle indices of triangles binned by warps
    uint32_t *large_count;   // 1
};

struct MeshDev {
    const float *x, *y, *z;  // nvert
    const uint32_t *idx;     // 3*ntri or nullptr (soup)
    const uint8_t *rgb;      // 3*ntri
    uint32_t nvert, ntri;
};

struct Mat4 {
    float m[16];             // row-major
};

// vertex transform: tv[i] = (M*v_i).xyz (nalgebra order), float4 per vertex.
cudaError_t launch_vertex_transform(const MeshDev &mesh, const Mat4 &M, float4 *tv,
                                    cudaStream_t s);

// per-triangle setup: records[tri_base + t], small-triangle tile counts and newline rows,
// large-triangle queue.
cudaError_t launch_setup(const MeshDev &mesh, const float4 *tv, uint32_t tri_base,
                         const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb,
                         cudaStream_t s);
// newline sentinels (image mode): fold each triangle's row range into the segment tree.
cudaError_t launch_newline(uint32_t ntri, uint32_t tri_base, const FrameGeom &g,
                           const FrameBuffers &fb, cudaStream_t s);
cudaError_t launch_bin_count_large(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                                   const BinBuffers &bb, cudaStream_t s);
cudaError_t launch_bin_scan(uint32_t ntiles, const BinBuffers &bb, cudaStream_t s);
cudaError_t launch_bin_fill(uint32_t ntri, uint32_t tri_base, const FrameGeom &g,
                            const FrameBuffers &fb, const BinBuffers &bb, cudaStream_t s);
cudaError_t launch_bin_fill_large(uint32_t tri_base, const FrameGeom &g, const FrameBuffers &fb,
                                  const BinBuffers &bb, cudaStream_t s);

// per-tile raster: 64-bit atomicMin of depth keys in shared memory, merged into keys.
cudaError_t launch_raster(const FrameGeom &g, const FrameBuffers &fb, const BinBuffers &bb, int depth_cull,
                          cudaStream_t s);

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
