/*
 * sloth_oracle.h -- CPU restatement of sloth's rasterization path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: a plain-C restatement of
 * the reference's sequential rasterizer, used by tests/, by smoke() and by the
 * bench's CPU-baseline leg.  The product library (libsloth_gpu.so) never links,
 * loads or calls it.
 *
 * Parity status: the reference is Rust and no Rust toolchain exists on either
 * machine, so the reference cannot be run.  The oracle is pinned against the
 * reference's own known-answer tests (src/geometry.rs:196-234) and against
 * hand-computed micro cases; the nalgebra 0.22.1 summation orders it assumes
 * (matrix products, vector norm) are not pinned by any reference test.
 *
 * Compiled with -O2 -ffp-contract=off -fno-fast-math: every float operation is
 * a separately rounded IEEE binary32 operation, as in Rust.
 */
#ifndef SLOTH_ORACLE_H
#define SLOTH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Frame cell packing shared with the GPU library: byte0 = ASCII char,
 * byte1 = r, byte2 = g, byte3 = b.  (' ', (0,0,0)) is 0x00000020. */
#define ORC_CELL(ch, r, g, b) \
    ((uint32_t)(uint8_t)(ch) | ((uint32_t)(r) << 8) | ((uint32_t)(g) << 16) | ((uint32_t)(b) << 24))

/* A render context: src/context.rs:12-19 (Context{utransform,width,height,
 * frame_buffer,z_buffer,image}).  Buffers are caller-owned. */
typedef struct {
    uint32_t width, height;
    int32_t image;          /* 1: image mode (w*h+h frame cells, newline sentinels) */
    float U[16];            /* utransform, row-major */
    float *z;               /* w*h */
    uint32_t *cells;        /* w*h (+h in image mode) */
    int32_t *winner;        /* optional (may be NULL): w*h, global triangle index of the
                               last accepted depth write, -1 when none */
    uint64_t fragments;     /* covered samples (all three edge functions >= 0) */
    uint64_t candidates;    /* samples visited by the loops */
    uint32_t next_tri;      /* global triangle counter since clear (draw order) */
    uint32_t *winner_xy;    /* optional (may be NULL): w*h, sample point x | y << 16 of the
                               last accepted depth write (differentiable shading's visibility) */
} orc_ctx;

/* src/rasterizer.rs:5-27 default_shader: shade -> ASCII ramp char. */
char orc_default_shader(float shade);

/* src/context.rs:35-45 Context::clear. */
void orc_clear(orc_ctx *ctx);

/* nalgebra 0.22.1 Matrix4*Matrix4 (gemm -> gemv column by column):
 * out[i][j] = ((A[i][0]*B[0][j] + A[i][1]*B[1][j]) + A[i][2]*B[2][j]) + A[i][3]*B[3][j]. */
void orc_mat4_mul(const float A[16], const float B[16], float out[16]);

/* nalgebra Matrix4*Vector4 with w = 1 (src/geometry.rs:43-48). */
void orc_mat4_vec(const float M[16], const float v[4], float out[4]);

/* nalgebra 0.22.1 Rotation3::from_euler_angles(roll, pitch, yaw).to_homogeneous()
 * (src/main.rs:76-77); row-major 4x4 out. */
void orc_euler_rotation(float roll, float pitch, float yaw, float out[16]);

/* src/context.rs:104-138 Context::update: the scene extent is the fold
 * 0.0.max(bbox.max.x).max(bbox.max.y).max(bbox.max.z) over meshes; bbox_max holds
 * 3 floats per mesh.  Writes the row-major utransform. */
float orc_scene_extent(const float *bbox_max, uint32_t nmesh);
void orc_viewport_transform(uint16_t width, uint16_t height, float extent, float U[16]);

/* Triangle methods of src/geometry.rs:36-57 on a triangle held as three Vector4
 * (v[0..3] = v1, v[4..7] = v2, v[8..11] = v3). */
void orc_triangle_mul(float v[12], const float M[16]);                   /* :43-48 */
void orc_triangle_aabb(const float v[12], float mn[4], float mx[4]);     /* :37-42 */
void orc_triangle_normal(const float v[12], float n[4]);                 /* :49-56 */

/* src/rasterizer.rs:48-93 draw_triangle.  v holds the triangle's three object-space
 * vertices (x,y,z each); M = utransform*transform (already multiplied, see
 * src/rasterizer.rs:57).  rgb = face colour.  Advances ctx->next_tri. */
void orc_draw_triangle(orc_ctx *ctx, const float v[9], const uint8_t rgb[3], const float M[16]);

/* src/rasterizer.rs:39-46 draw_mesh over an SoA mesh.  x,y,z: vertex positions;
 * idx: 3 u32 per triangle, or NULL for an unindexed soup (vertex 3t+k);
 * rgb: 3 u8 per triangle.  R = the rotation ("transform"); the product
 * utransform*R is formed once (it is the same value for every triangle). */
void orc_draw_mesh(orc_ctx *ctx, const float *x, const float *y, const float *z,
                   const uint32_t *idx, const uint8_t *rgb, uint32_t ntri, const float R[16]);

/* Same sequential algorithm, split over `nthreads` threads by target-row bands so the
 * CPU baseline can use every host core.  Each band owns the depth cells of its rows and
 * the frame cells of its rows; every band visits the triangles in draw order, so every
 * cell sees exactly the reference's write sequence.  Results are identical to
 * orc_draw_mesh.  Fragment/candidate counters are summed over bands. */
void orc_draw_mesh_banded(orc_ctx *ctx, const float *x, const float *y, const float *z,
                          const uint32_t *idx, const uint8_t *rgb, uint32_t ntri,
                          const float R[16], int nthreads);

#ifdef __cplusplus
}
#endif
/* src/context.rs:50-92 Context::flush(color, webify): the bytes written to stdout for a
 * frame of cells (char | r<<8 | g<<16 | b<<24).  format 0: color false (chars, then
 * println's newline); 1: color true, webify false (per cell crossterm 0.18's styled char:
 * ESC[48;2;25;25;25m ESC[38;2;r;g;bm char ESC[0m); 2: color true, webify true (per cell
 * <span style="color:rgb(r,g,b)">char).  A terminal context (image 0) starts with
 * crossterm's MoveTo(0,0) = ESC[1;1H.  out may be NULL (size only); returns the size. */
uint64_t orc_flush(const uint32_t *cells, uint64_t ncells, int image, int format, char *out);

#endif
