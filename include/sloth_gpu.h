/*
 * sloth_gpu.h -- C ABI of the GB300 rasterization path for sloth (ecumene/rust-sloth).
 *
 * The library replaces the body of sloth's per-frame draw path:
 *   Context::clear      src/context.rs:35-45
 *   Context::update     src/context.rs:93-141   (the viewport transform, host math)
 *   draw_mesh           src/rasterizer.rs:39-46  (-> draw_triangle :48-93, default_shader :5-27)
 *   frame_buffer/z_buffer read-back (what Context::flush prints, src/context.rs:50-92)
 * and keeps the reference's results bit for bit: depth cells, frame cells (char and
 * colour), the newline sentinels of image mode and the draw-order tie-break.
 *
 * Conventions
 *  - Plain C types, caller-owned host buffers, library-owned device buffers.
 *  - Every fallible call returns sloth_status; sloth_ctx_last_error() gives the text.
 *    Nothing panics or throws across the ABI.
 *  - One CUDA stream per context (caller-supplied or library-created); calls on one
 *    context are not thread-safe, like the reference's &mut Context.
 *  - Matrices are row-major float[16] (nalgebra's Matrix4::new argument order).
 *  - A frame cell is a uint32: byte0 = ASCII char, byte1 = r, byte2 = g, byte3 = b.
 *    The reference's (char,(u8,u8,u8)) cell; all chars it produces are ASCII.
 *  - The shader is fixed to default_shader (a Rust closure cannot cross a C ABI);
 *    its thresholds are exported by sloth_shader_thresholds().
 */
#ifndef SLOTH_GPU_H
#define SLOTH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sloth_status {
    SLOTH_OK = 0,
    SLOTH_ERR_INVALID_ARGUMENT = 1,
    SLOTH_ERR_OUT_OF_MEMORY = 2,
    SLOTH_ERR_CUDA = 3,
    SLOTH_ERR_LIMIT = 4,          /* a size beyond a documented limit */
    SLOTH_ERR_DEVICE_FAULT = 5    /* a kernel gave up waiting for one of its copies (reported
                                     by the next synchronising call; the frame is invalid) */
} sloth_status;

typedef struct sloth_ctx sloth_ctx;
typedef struct sloth_mesh sloth_mesh;

/* Limits of this implementation. */
#define SLOTH_MAX_DIM 65535u              /* width/height: the reference casts them to u16 in update */
#define SLOTH_MAX_TRIANGLES 0x7fffffffu   /* triangles drawn between two clears (31-bit draw index) */

/* ---- library ---------------------------------------------------------------------- */

/* Version string of this library. */
const char *sloth_version(void);

/* default_shader's ramp (src/rasterizer.rs:5-27): thresholds[9] = 0.2f..1.0f and
 * chars[10] = ".:-=+*#%@ " (the last char is used above 1.0 and for NaN). */
void sloth_shader_thresholds(float thresholds[9], char chars[10]);

/* default_shader itself, evaluated on the host (src/rasterizer.rs:5-27). */
char sloth_default_shader(float shade);

/* ---- host math the reference does before drawing ---------------------------------- */

/* nalgebra 0.22.1 Rotation3::from_euler_angles(roll, pitch, yaw).to_homogeneous(),
 * as built per frame at src/main.rs:76-77.  out: row-major 4x4. */
void sloth_euler_rotation(float roll, float pitch, float yaw, float out[16]);

/* nalgebra Matrix4 * Matrix4 (src/rasterizer.rs:57 utransform*transform), with its
 * column-by-column, left-to-right accumulation order. */
void sloth_mat4_mul(const float a[16], const float b[16], float out[16]);

/* The scene extent of Context::update (src/context.rs:106-113): the fold
 * 0.0.max(bbox.max.x).max(bbox.max.y).max(bbox.max.z) over meshes.
 * bbox_max: 3 floats per mesh. */
float sloth_scene_extent(const float *bbox_max, uint32_t nmesh);

/* The utransform of Context::update (src/context.rs:114-133) for a width x height
 * context and a scene extent.  out: row-major 4x4. */
void sloth_viewport_transform(uint16_t width, uint16_t height, float extent, float out[16]);

/* The order in which setup takes an indexed mesh's triangles (host only, no device
 * needed): order[p] is the triangle at position p, by ascending Morton code (10 bits an
 * axis, x in the lowest bit) of its centroid's place in the box of the finite centroids,
 * ties in index order, a non-finite centroid taking code 0.  sloth_mesh_create makes it
 * for every indexed mesh; the results of a draw do not depend on it.  x, y, z: nvert
 * vertex positions; idx: 3*ntri indices; order: ntri outputs.  SLOTH_ERR_INVALID_ARGUMENT
 * for NULL arrays or an index not below nvert, SLOTH_ERR_OUT_OF_MEMORY without host
 * memory for the sort. */
sloth_status sloth_spatial_order(const float *x, const float *y, const float *z, uint32_t nvert, const uint32_t *idx,
                                 uint32_t ntri, uint32_t *order);

/* ---- context (src/context.rs:12-49) ------------------------------------------------- */

/* Create a context on CUDA device `device`.  `stream` is a cudaStream_t to order all
 * work on, or NULL for a library-owned stream: a draw forks two kernels onto the
 * context's own helper streams (the newline fold, the large-triangle fill) and joins
 * them back into `stream` before the draw's raster, the resolve, the next draw and
 * sloth_ctx_synchronize, so results read from `stream` are complete.  The context starts
 * blank like Context::blank(image=false) (src/context.rs:22-34): 0x0 viewport, identity
 * utransform.  Contexts are independent: different host threads may drive different
 * contexts at once. */
sloth_status sloth_ctx_create(sloth_ctx **out, int device, void *stream);
/* Destroys the context.  Batches made on it lose their device memory; they and the
 * context's meshes stay valid handles only for sloth_batch_destroy / sloth_mesh_destroy
 * (a mesh also keeps drawing on other contexts of its device). */
void sloth_ctx_destroy(sloth_ctx *ctx);

/* Text of the last error on this context ("" when none). */
const char *sloth_ctx_last_error(const sloth_ctx *ctx);

/* Set width, height and image mode (Context{width,height,image}; match_dimensions,
 * src/inputs.rs:159-169, or the terminal size).  image != 0 gives w*h+h frame cells
 * with newline sentinels (src/context.rs:36-42, src/rasterizer.rs:89-91).
 * 1 <= width,height <= SLOTH_MAX_DIM.  Takes effect at the next clear. */
sloth_status sloth_ctx_set_viewport(sloth_ctx *ctx, uint32_t width, uint32_t height, int image);

/* Set the utransform directly (Context.utransform / Context::camera, src/context.rs:46-49). */
sloth_status sloth_ctx_set_utransform(sloth_ctx *ctx, const float u[16]);

/* Context::update (src/context.rs:93-141) for image mode: utransform from the meshes'
 * bounding boxes and the current viewport. */
sloth_status sloth_ctx_update(sloth_ctx *ctx, const sloth_mesh *const *meshes, uint32_t nmesh);

/* Context::clear (src/context.rs:35-45): depth <- f32::MAX, frame <- (' ',(0,0,0)),
 * and the draw-order counter restarts. */
sloth_status sloth_ctx_clear(sloth_ctx *ctx);

/* Number of frame cells (w*h, or w*h+h in image mode) and depth cells (w*h). */
sloth_status sloth_ctx_sizes(const sloth_ctx *ctx, uint64_t *frame_cells, uint64_t *depth_cells);

/* Copy the frame (Context.frame_buffer) and depth (Context.z_buffer) buffers to host
 * memory; any argument may be NULL.  `winner` (w*h int32) receives the draw index of
 * the triangle that last passed the depth test at each depth cell, or -1.
 * Blocks until the copies complete. */
sloth_status sloth_ctx_read(sloth_ctx *ctx, uint32_t *cells, float *z, int32_t *winner);

/* sloth_ctx_read without waiting: the copies are queued on the context's stream (host
 * buffers should be page-locked) and complete by the next sloth_ctx_synchronize.  With
 * two contexts used in turn, one frame's read-back overlaps the next frame's upload and
 * draw.  Not in the reference, whose Context is synchronous. */
sloth_status sloth_ctx_read_async(sloth_ctx *ctx, uint32_t *cells, float *z, int32_t *winner);
/* Wait for everything queued on the context's stream. */
sloth_status sloth_ctx_synchronize(sloth_ctx *ctx);

/* Device pointers of the resolved buffers (valid until the next clear/resize/destroy),
 * for consumers that stay on the GPU.  Resolves pending draws first (asynchronously). */
sloth_status sloth_ctx_device_buffers(sloth_ctx *ctx, const uint32_t **cells, const float **z);

/* Covered samples (all three edge functions >= 0, src/rasterizer.rs:75) since the last
 * clear, counted by the raster kernels over the triangles they evaluated: every covered
 * sample when SLOTH_OPTION_DEPTH_CULL is 0.  Blocks until pending work completes. */
sloth_status sloth_ctx_fragments(sloth_ctx *ctx, uint64_t *fragments);

/* The bytes Context::flush(color, webify) prints for the frame (src/context.rs:50-92),
 * formatted on the GPU from the resolved frame cells:
 *   SLOTH_FLUSH_PLAIN  color false: every char, then "\n" (println);
 *   SLOTH_FLUSH_ANSI   color true, webify false: per cell crossterm's styled char,
 *                      ESC[48;2;25;25;25m ESC[38;2;<r>;<g>;<b>m <char> ESC[0m;
 *   SLOTH_FLUSH_HTML   color true, webify true: per cell <span style="color:rgb(<r>,<g>,<b>)"><char>.
 * A terminal context (image 0) starts with crossterm's MoveTo(0,0), ESC[1;1H.  The ANSI
 * form restates crossterm 0.18.0 (the version the reference's Cargo.lock pins), whose
 * source is not part of the reference.
 * sloth_ctx_flush: *bytes = the size; with out != NULL the bytes are copied there
 * (SLOTH_ERR_LIMIT if capacity < size).  Blocks.
 * sloth_ctx_flush_device: the bytes stay on the device (valid until the next flush of the
 * context or its destruction). */
#define SLOTH_FLUSH_PLAIN 0
#define SLOTH_FLUSH_ANSI 1
#define SLOTH_FLUSH_HTML 2
sloth_status sloth_ctx_flush(sloth_ctx *ctx, int format, char *out, uint64_t capacity, uint64_t *bytes);
sloth_status sloth_ctx_flush_device(sloth_ctx *ctx, int format, const char **device_bytes, uint64_t *bytes);

/* Options (sloth_ctx_set_option).
 * SLOTH_OPTION_DEPTH_CULL: 1 (default) lets the raster skip triangles proven to lie
 *   behind every depth cell they could write (a proven depth bound against the tile's
 *   current depths); 0 rasterizes every triangle.  Results are identical either way. */
#define SLOTH_OPTION_DEPTH_CULL 1
/* SLOTH_OPTION_TILE_SHAPE: index of the raster's tile shape (see sloth_tile_shape; 0 is
 *   64 cells x 32 rows); takes effect at the next sloth_ctx_clear. */
#define SLOTH_OPTION_TILE_SHAPE 2
/* SLOTH_OPTION_WAIT_TEST: a test hook.  1 makes every raster block that loads keys of an
 *   earlier draw wait, with a short limit, for 16 bytes that never arrive; the block gives
 *   up, leaves its tile as it is and the next synchronising call returns
 *   SLOTH_ERR_DEVICE_FAULT (a clear starts the next frame without the error).  0 (the
 *   default) is normal operation. */
#define SLOTH_OPTION_WAIT_TEST 3
/* SLOTH_OPTION_DIRECT_SAMPLES: triangles whose sample range (after the exact tightening of
 *   its right edge) holds at most this many samples are rasterized by the setup kernel
 *   straight into the global depth keys (a 64-bit atomicMin per covered sample) instead of
 *   being binned into tiles; 0 (the default) bins every triangle.  0..SLOTH_MAX_DIRECT_SAMPLES;
 *   takes effect at the next sloth_ctx_clear.  Results are identical either way. */
#define SLOTH_OPTION_DIRECT_SAMPLES 4
#define SLOTH_MAX_DIRECT_SAMPLES 256
/* SLOTH_OPTION_TRIANGLES_PER_BLOCK: triangles per block of the setup kernel, 128, 256 (the
 *   default), 1024 or 4096; a block has at most 256 threads, each taking its share of the
 *   block's triangles in turn.  Results are identical either way. */
#define SLOTH_OPTION_TRIANGLES_PER_BLOCK 5
sloth_status sloth_ctx_set_option(sloth_ctx *ctx, int option, int64_t value);

/* Autotuner of the single-frame path: renders the frame clear + draw_mesh(meshes[i],
 * transforms[16*i]) for i < ndraws + resolve, `reps` times per candidate setting, and keeps
 * the fastest (tile shape, direct-sample limit in {0, 4, 16, 64}, triangles per block in
 * {128, 256, 1024, 4096}) as the context's options; reports them and the mean frame time in ms
 * (any output may be NULL).  Needs a viewport and utransform; leaves the context with the
 * last candidate's frame drawn (clear before the next frame). */
sloth_status sloth_ctx_autotune(sloth_ctx *ctx, const sloth_mesh *const *meshes, const float *transforms,
                                uint32_t ndraws, int reps, int *best_shape, int *best_direct, int *best_tpb,
                                float *best_ms);

/* The raster tile shapes the library is built for: shape i is `cells` depth cells wide
 * and `rows` rows high; SLOTH_ERR_INVALID_ARGUMENT past the last shape. */
sloth_status sloth_tile_shape(int shape, uint32_t *cells, uint32_t *rows);

/* ---- meshes (SimpleMesh, src/geometry.rs:78-81) ------------------------------------ */

/* Upload a mesh to the context's device.  x,y,z: nvert vertex positions (structure of
 * arrays).  idx: 3*ntri vertex indices, or NULL for an unindexed triangle soup
 * (triangle t uses vertices 3t, 3t+1, 3t+2; then nvert must be 3*ntri).  rgb: 3*ntri
 * face colours (Triangle.color).  bbox_max: the SimpleMesh bounding_box.max (x,y,z) that
 * Context::update folds, or NULL to use the loader rule of OBJ meshes
 * (src/geometry.rs:86-89,128-135: a box grown from the origin).  An indexed mesh also
 * gets the order in which setup takes its triangles (a Morton order of their centroids,
 * sorted on the host here, 16 more device bytes a triangle); draws still follow the
 * mesh's own triangle order, which the results depend on, not that one. */
sloth_status sloth_mesh_create(sloth_ctx *ctx, const float *x, const float *y, const float *z,
                               uint32_t nvert, const uint32_t *idx, uint32_t ntri,
                               const uint8_t *rgb, const float *bbox_max, sloth_mesh **out);
void sloth_mesh_destroy(sloth_mesh *mesh);

/* Overwrite a mesh's vertex positions and face colours in place (same nvert/ntri), with
 * asynchronous copies on the context's stream; page-locked host buffers make them true
 * async copies.  The sources may be host or device memory (unified addressing decides
 * the copy direction).  The buffers must stay valid until the next synchronising call. */
sloth_status sloth_mesh_update(sloth_mesh *mesh, const float *x, const float *y, const float *z,
                               const uint8_t *rgb);
sloth_status sloth_mesh_info(const sloth_mesh *mesh, uint32_t *ntri, float bbox_max[3]);

/* ---- the hot path ----------------------------------------------------------------- */

/* draw_mesh(context, mesh, transform, default_shader) (src/rasterizer.rs:39-46): draws
 * every triangle of `mesh` in order, after all triangles drawn since the last clear.
 * transform: the row-major rotation (or any model matrix); the library forms
 * utransform*transform once, in nalgebra's order.  Asynchronous on the ctx stream: the
 * host does not wait for the GPU, except on the context's first draw (which sizes the
 * tile-entry buffer from its count) and when a buffer grows.  A draw whose tile entries
 * outgrow the entry buffer is rasterized by a slower exact fallback on the device, and a
 * later draw grows the buffer. */
sloth_status sloth_draw_mesh(sloth_ctx *ctx, const sloth_mesh *mesh, const float transform[16]);

/* ---- many frames at once --------------------------------------------------------- */

/* The reference renders frame after frame (src/main.rs:60-111: update, clear, draw every
 * mesh of the queue, flush); its multi-frame JS export (`image -j N`, src/main.rs:55-58,
 * 92-106) and multi-model queues (src/inputs.rs:95-129) repeat that loop.  A batch holds
 * many such frames -- views, meshes and viewports of uneven sizes -- and renders all of
 * them with one pass of each stage and one persistent raster pass over a device-side
 * (frame, tile) queue, replayed as a CUDA graph.  Every frame is bit-identical to
 * clear + draw_mesh of its draws in order on a context with the same viewport. */
typedef struct sloth_batch sloth_batch;

typedef struct sloth_draw_desc {
    const sloth_mesh *mesh;    /* draw_mesh(context, mesh, transform, default_shader) */
    float transform[16];       /* row-major */
} sloth_draw_desc;

typedef struct sloth_frame_desc {
    uint32_t width, height;    /* Context.width/height */
    int32_t image;             /* Context.image */
    float utransform[16];      /* Context.utransform, row-major */
    uint32_t first_draw;       /* the frame draws draws[first_draw .. first_draw+ndraws) in order; */
    uint32_t ndraws;           /* frames list consecutive ranges starting at draw 0 */
} sloth_frame_desc;

/* Lay out a batch on the context's device and stream (the meshes must outlive it). */
sloth_status sloth_batch_create(sloth_ctx *ctx, const sloth_frame_desc *frames, uint32_t nframes,
                                const sloth_draw_desc *draws, uint32_t ndraws, sloth_batch **out);
void sloth_batch_destroy(sloth_batch *batch);
/* Replace every draw's transform (16 floats per draw); waits for the previous render. */
sloth_status sloth_batch_set_transforms(sloth_batch *batch, const float *transforms);
/* Render every frame (asynchronous on the context's stream).  The first render sizes the
 * tile-entry buffer (one host synchronisation); later renders replay a CUDA graph. */
sloth_status sloth_batch_render(sloth_batch *batch);
/* Copy one frame's buffers to host memory (any may be NULL); blocks.  If the last render
 * outgrew the tile-entry buffer, it is re-planned and re-rendered first. */
sloth_status sloth_batch_read(sloth_batch *batch, uint32_t frame, uint32_t *cells, float *z, int32_t *winner);
/* Device pointers of one frame's resolved buffers. */
sloth_status sloth_batch_frame_buffers(sloth_batch *batch, uint32_t frame, const uint32_t **cells,
                                       const float **z);
/* Fragments the raster evaluated in the last render, summed over frames (see
 * sloth_ctx_fragments); blocks. */
sloth_status sloth_batch_fragments(sloth_batch *batch, uint64_t *fragments);
/* sloth_ctx_flush for one frame of the batch. */
sloth_status sloth_batch_flush(sloth_batch *batch, uint32_t frame, int format, char *out, uint64_t capacity,
                               uint64_t *bytes);
/* Use tile shape `shape` (sloth_tile_shape) for this batch; re-lays out its buffers. */
sloth_status sloth_batch_set_tile_shape(sloth_batch *batch, int shape);
/* persistent != 0 (the default): the raster is a grid of SMs x resident CTAs that take
 * (frame, tile) items from a device-side queue until it is empty; 0: one CTA per item,
 * balanced by the hardware block scheduler.  The frames are the same either way. */
sloth_status sloth_batch_set_persistent(sloth_batch *batch, int persistent);
/* Rasterize triangles of at most `samples` samples straight into the depth keys during
 * setup (SLOTH_OPTION_DIRECT_SAMPLES for a batch; a new batch takes its context's value). */
sloth_status sloth_batch_set_direct_samples(sloth_batch *batch, int samples);
/* Triangles per block of the batch's setup kernel (SLOTH_OPTION_TRIANGLES_PER_BLOCK):
 * 128, 256 (the default), 1024 or 4096. */
sloth_status sloth_batch_set_triangles_per_block(sloth_batch *batch, int tpb);
/* Autotuner: times `reps` renders of the batch per candidate setting and keeps the fastest
 * (tile shape, direct-sample limit in {0, 4, 16, 64}, triangles per block in {128, 256,
 * 1024, 4096}, persistent raster or not), searching one dimension at a time from the current
 * settings, twice over; reports the choice and its mean render time in ms (any output may
 * be NULL).  Every setting renders the same frames. */
sloth_status sloth_batch_autotune(sloth_batch *batch, int reps, int *best_shape, int *best_direct, int *best_tpb,
                                  int *best_persistent, float *best_ms);

/* ---- differentiable shading of a rendered batch ----------------------------------- */

/* No counterpart in the reference, which only maps the screen-space normal's z to a
 * character (src/rasterizer.rs:76, default_shader at src/rasterizer.rs:5-27).  These
 * calls define a smooth f32 image on the visibility of the last render and its adjoint,
 * for fitting a mesh to images (inverse rendering).
 *
 * Every draw of the batch must use one mesh.  For the winning sample (x, y) of depth
 * cell c of a frame (the triangle whose depth key won the cell, as in the render), with
 * A, B, C that triangle's vertices after the draw's utransform*transform:
 *     rgb[c] = (b0*col(A) + b1*col(B) + b2*col(C)) * clamp(n . L, 0, 1)
 * b_i the barycentric weights of (x, y) in the 2-D triangle (ABC), n the unit normal of
 * (B-A) x (C-A), col the per-vertex colour (vertex_rgb, 3 floats per mesh vertex) and L
 * the light direction in screen space (L = (0,0,1) makes the shade factor the
 * reference's normal z).  Cells without a winner, and zero-area triangles, give 0.
 * Visibility (which triangle and sample) is piecewise constant in the vertex positions
 * and is not differentiated.
 *
 * rgb holds 3 floats per depth cell of every frame, frames in order
 * (sloth_batch_depth_cells gives a frame's offset and size, in cells).  vertex_rgb, light
 * (3 floats), rgb and every gradient buffer are device memory; calls are asynchronous on
 * the context's stream.  With store_visibility = 1 the forward call also keeps the
 * winning (triangle, sample) of every cell (8 bytes per depth cell) for the next backward
 * call; otherwise the backward call decodes it again from the depth keys.  Either way the
 * backward call must follow the render it differentiates, before the next render. */
sloth_status sloth_batch_depth_cells(sloth_batch *batch, uint32_t frame, uint64_t *first, uint64_t *count);
sloth_status sloth_batch_shade(sloth_batch *batch, const float *vertex_rgb, const float *light, float *rgb,
                               int store_visibility);
/* Adds d(loss)/d(vertex position) (3 floats per mesh vertex, object space, i.e. the x, y,
 * z arrays of sloth_mesh_create/update), d(loss)/d(vertex_rgb) and d(loss)/d(light) to
 * grad_pos, grad_vertex_rgb and grad_light (any may be NULL), for grad_rgb =
 * d(loss)/d(rgb).  The sums use float atomics, so their last bits vary run to run. */
sloth_status sloth_batch_shade_backward(sloth_batch *batch, const float *vertex_rgb, const float *light,
                                        const float *grad_rgb, float *grad_pos, float *grad_vertex_rgb,
                                        float *grad_light);

/* ---- one frame without device allocation ------------------------------------------ */

/* No counterpart in the reference.  For callers that cannot let a library allocate
 * device memory: hosts that fix the renderer's memory at start-up and forbid allocation
 * afterwards, frame loops that cannot afford the device-wide synchronisation of
 * cudaMalloc/cudaFree, and programs whose memory is held by a framework's caching pool.
 *
 * Draws one unindexed triangle soup (triangle t = vertices 3t..3t+2 of x, y, z; face
 * colours rgb, 3 per triangle) into a cleared width x height context and writes its
 * frame cells (cells: w*h, or w*h+h in image mode), depth buffer (zbuf: w*h) and winners
 * (winner: w*h) -- the same values as sloth_ctx_clear + sloth_draw_mesh + sloth_ctx_read.
 * m = utransform*transform, row-major, in host memory.  Every other pointer is device
 * memory owned by the caller.  Work is queued on `stream` (a cudaStream_t, NULL = the
 * default stream); the call returns without waiting for it.
 *
 * It calls no cudaMalloc or cudaFree: all intermediate buffers live in one __device__
 * array of SLOTH_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library holds
 * until the process exits.  Limits: ntri <= SLOTH_NOALLOC_MAX_TRIANGLES,
 * height <= SLOTH_NOALLOC_MAX_HEIGHT, and the viewport padded to 64x32-cell tiles
 * ((ceil(w/64)*64) * (ceil(h/32)*32)) <= SLOTH_NOALLOC_MAX_DEPTH_CELLS; larger inputs
 * return SLOTH_ERR_LIMIT.  Every call looks up the array's device address
 * (cudaGetSymbolAddress, which allocates nothing) on the device the caller made current,
 * so an address never outlives a cudaDeviceReset; the first call on a device also loads
 * the library's kernels there, so make that first call before any stream capture.  All
 * calls share the array, so calls that overlap on the GPU (on different streams, or from
 * different threads) race and corrupt each other's frames: issue them one after another. */
#define SLOTH_NOALLOC_MAX_TRIANGLES 32768u
#define SLOTH_NOALLOC_MAX_HEIGHT 4096u
#define SLOTH_NOALLOC_MAX_DEPTH_CELLS 524288u
#define SLOTH_NOALLOC_SCRATCH_BYTES 7639808u
sloth_status sloth_render_noalloc(const float *x, const float *y, const float *z, uint32_t ntri,
                                  const uint8_t *rgb, const float m[16], uint32_t width,
                                  uint32_t height, int image, uint32_t *cells, float *zbuf,
                                  int32_t *winner, void *stream);

/* ---- timing hooks for benchmarks -------------------------------------------------- */

/* Enable (1) / disable (0) CUDA-event timing of each kernel the context launches.
 * sloth_ctx_kernel_time() then reports the summed device time (ms) and launch count
 * of kernel `name` ("setup", "bin_count_large", "bin_scan", "bin_fill", "bin_fill_large",
 * "bin_items", "raster", "resolve") since timing was enabled; blocks until the events complete. */
sloth_status sloth_ctx_set_timing(sloth_ctx *ctx, int enable);
sloth_status sloth_ctx_kernel_time(sloth_ctx *ctx, const char *name, double *ms, uint64_t *launches);
/* Number of kernels launched by this context since creation. */
uint64_t sloth_ctx_launch_count(const sloth_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
