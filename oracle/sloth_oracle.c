/*
 * sloth_oracle.c -- CPU restatement of sloth's rasterization path.
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle and the CPU baseline).  Nothing in
 * the product library links or calls this file.
 *
 * Each function cites the reference line it restates (paths relative to the
 * ecumene/rust-sloth tree).  Float arithmetic keeps the reference's operation
 * order; the file must be compiled with -ffp-contract=off -fno-fast-math so that
 * no multiply-add is fused (Rust never contracts).
 *
 * Third-party arithmetic restated here (not present in the reference tree):
 *  - nalgebra 0.22.1 (Cargo.lock): Matrix4*Matrix4 and Matrix4*Vector4 go through
 *    gemm -> gemv -> axcpy, which accumulates column by column, left to right,
 *    starting from the first product (no leading zero add).  Vector4::norm() goes
 *    through dotx, which special-cases 4-vectors as (a*a + c*c) + (b*b + d*d).
 *    Unit::new_normalize divides each component by the norm.
 *    Rotation3::from_euler_angles(roll, pitch, yaw) builds the ZYX product
 *    [[cy*cp, cy*sp*sr - sy*cr, cy*sp*cr + sy*sr],
 *     [sy*cp, sy*sp*sr + cy*cr, sy*sp*cr - cy*sr],
 *     [-sp,   cp*sr,            cp*cr]] with (s,c) = sin_cos of each angle.
 *  No reference test pins these orders (the known-answer tests at
 *  src/geometry.rs:196-234 use exactly representable values).
 */
#include "sloth_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_FLT_MAX 3.40282347e+38f

/* src/rasterizer.rs:5-27 */
char orc_default_shader(float shade)
{
    if (shade <= 0.20f) return '.';
    else if (shade <= 0.30f) return ':';
    else if (shade <= 0.40f) return '-';
    else if (shade <= 0.50f) return '=';
    else if (shade <= 0.60f) return '+';
    else if (shade <= 0.70f) return '*';
    else if (shade <= 0.80f) return '#';
    else if (shade <= 0.90f) return '%';
    else if (shade <= 1.0f) return '@';
    return ' ';
}

/* src/context.rs:35-45 */
void orc_clear(orc_ctx *ctx)
{
    uint64_t n = (uint64_t)ctx->width * ctx->height;
    uint64_t ncells = ctx->image ? n + ctx->height : n;
    for (uint64_t i = 0; i < ncells; ++i) ctx->cells[i] = ORC_CELL(' ', 0, 0, 0);
    for (uint64_t i = 0; i < n; ++i) ctx->z[i] = ORC_FLT_MAX;
    if (ctx->winner)
        for (uint64_t i = 0; i < n; ++i) ctx->winner[i] = -1;
    if (ctx->winner_xy)
        for (uint64_t i = 0; i < n; ++i) ctx->winner_xy[i] = 0xffffffffu;
    ctx->fragments = 0;
    ctx->candidates = 0;
    ctx->next_tri = 0;
}

/* nalgebra gemm/gemv order (used at src/rasterizer.rs:57). */
void orc_mat4_mul(const float A[16], const float B[16], float out[16])
{
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float acc = A[i * 4 + 0] * B[0 * 4 + j];
            acc = A[i * 4 + 1] * B[1 * 4 + j] + acc;
            acc = A[i * 4 + 2] * B[2 * 4 + j] + acc;
            acc = A[i * 4 + 3] * B[3 * 4 + j] + acc;
            r[i * 4 + j] = acc;
        }
    memcpy(out, r, sizeof r);
}

/* src/geometry.rs:43-48 Triangle::mul, one vertex. */
void orc_mat4_vec(const float M[16], const float v[4], float out[4])
{
    float r[4];
    for (int i = 0; i < 4; ++i) {
        float acc = M[i * 4 + 0] * v[0];
        acc = M[i * 4 + 1] * v[1] + acc;
        acc = M[i * 4 + 2] * v[2] + acc;
        acc = M[i * 4 + 3] * v[3] + acc;
        r[i] = acc;
    }
    memcpy(out, r, sizeof r);
}

/* src/main.rs:76-77 (nalgebra Rotation3::from_euler_angles + to_homogeneous). */
void orc_euler_rotation(float roll, float pitch, float yaw, float out[16])
{
    float sr = sinf(roll), cr = cosf(roll);
    float sp = sinf(pitch), cp = cosf(pitch);
    float sy = sinf(yaw), cy = cosf(yaw);
    float m[16] = {
        cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr, 0.0f,
        sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr, 0.0f,
        -sp,     cp * sr,                cp * cr,                0.0f,
        0.0f,    0.0f,                   0.0f,                   1.0f,
    };
    memcpy(out, m, sizeof m);
}

/* src/context.rs:106-113: scale = 0.0; scale = scale.max(x).max(y).max(z) per mesh.
 * Rust's f32::max ignores a NaN operand, like fmaxf. */
float orc_scene_extent(const float *bbox_max, uint32_t nmesh)
{
    float s = 0.0f;
    for (uint32_t m = 0; m < nmesh; ++m) {
        s = fmaxf(s, bbox_max[3 * m + 0]);
        s = fmaxf(s, bbox_max[3 * m + 1]);
        s = fmaxf(s, bbox_max[3 * m + 2]);
    }
    return s;
}

/* src/context.rs:114-133 */
void orc_viewport_transform(uint16_t width, uint16_t height, float extent, float U[16])
{
    float fw = (float)width, fh = (float)height;
    float scale = fminf(fh, fw / 2.0f) / extent / 2.0f;
    float t[16] = {
        scale, 0.0f,   0.0f,  fw / 4.0f,
        0.0f,  -scale, 0.0f,  fh / 2.0f,
        0.0f,  0.0f,   scale, 0.0f,
        0.0f,  0.0f,   0.0f,  1.0f,
    };
    memcpy(U, t, sizeof t);
}

/* src/rasterizer.rs:30-32 */
static inline float orient(float ax, float ay, float bx, float by, float cx, float cy)
{
    return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
}

/* Rust `f as usize`: saturating, NaN -> 0. */
static inline uint64_t sat_usize(float f)
{
    if (!(f > 0.0f)) return 0;
    if (f >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)f;
}

/* Per-triangle setup shared by the sequential and the banded loops:
 * src/rasterizer.rs:56-67 and src/geometry.rs:37-56. */
typedef struct {
    float v[3][3];          /* transformed vertices (x,y,z) */
    float a;                /* 1 / orient(v1,v2,v3) */
    float nz;               /* normal().z */
    uint64_t x0, x1, y0, y1;
    uint8_t rgb[3];
    uint32_t tri;           /* global draw-order index */
} orc_setup;

/* src/geometry.rs:43-48 */
void orc_triangle_mul(float v[12], const float M[16])
{
    for (int k = 0; k < 3; ++k) orc_mat4_vec(M, &v[4 * k], &v[4 * k]);
}

/* src/geometry.rs:37-42: Vector4::from_fn(|x| v1[x].min(v2[x].min(v3[x]))), same for max. */
void orc_triangle_aabb(const float v[12], float mn[4], float mx[4])
{
    for (int c = 0; c < 4; ++c) {
        mn[c] = fminf(v[c], fminf(v[4 + c], v[8 + c]));
        mx[c] = fmaxf(v[c], fmaxf(v[4 + c], v[8 + c]));
    }
}

/* src/geometry.rs:49-56: cross product of v2-v1 and v3-v1 as a Vector4 with w = 0,
 * then Unit::new_normalize (norm via nalgebra's 4-vector dot, each component / norm). */
void orc_triangle_normal(const float v[12], float n[4])
{
    float e1[4], e2[4];
    for (int c = 0; c < 4; ++c) {
        e1[c] = v[4 + c] - v[c];
        e2[c] = v[8 + c] - v[c];
    }
    float x = (e1[1] * e2[2]) - (e1[2] * e2[1]);
    float y = (e1[2] * e2[0]) - (e1[0] * e2[2]);
    float z = (e1[0] * e2[1]) - (e1[1] * e2[0]);
    float w = 0.0f;
    float norm2 = (x * x + z * z) + (y * y + w * w);
    float len = sqrtf(0.0f + norm2);
    n[0] = x / len;
    n[1] = y / len;
    n[2] = z / len;
    n[3] = w / len;
}

static void triangle_setup(const orc_ctx *ctx, const float v[9], const uint8_t rgb[3],
                           const float M[16], uint32_t tri, orc_setup *s)
{
    /* dist_triangle = triangle.clone(); dist_triangle.mul(M)  (src/rasterizer.rs:56-57) */
    float tv[12];
    for (int k = 0; k < 3; ++k) {
        tv[4 * k + 0] = v[3 * k + 0];
        tv[4 * k + 1] = v[3 * k + 1];
        tv[4 * k + 2] = v[3 * k + 2];
        tv[4 * k + 3] = 1.0f;
    }
    orc_triangle_mul(tv, M);
    float mn[4], mx[4];
    orc_triangle_aabb(tv, mn, mx);
    /* src/rasterizer.rs:59-66 */
    s->x0 = sat_usize(ceilf(fmaxf(mn[0], 1.0f)));
    s->y0 = sat_usize(ceilf(fmaxf(mn[1], 1.0f)));
    s->x1 = sat_usize(ceilf(fminf(mx[0] * 2.0f, (float)(ctx->width - 1))));
    s->y1 = sat_usize(ceilf(fminf(mx[1], (float)(ctx->height - 1))));
    /* src/rasterizer.rs:67 */
    s->a = 1.0f / orient(tv[0], tv[1], tv[4], tv[5], tv[8], tv[9]);
    /* normal().z, used at src/rasterizer.rs:76 (the same value for every sample) */
    float n[4];
    orc_triangle_normal(tv, n);
    s->nz = n[2];
    for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 3; ++c) s->v[k][c] = tv[4 * k + c];
    s->rgb[0] = rgb[0]; s->rgb[1] = rgb[1]; s->rgb[2] = rgb[2];
    s->tri = tri;
}

/* The body of one sample, src/rasterizer.rs:71-86.  Returns 1 if covered. */
static inline int sample(orc_ctx *ctx, const orc_setup *s, uint64_t x, uint64_t y,
                         float *zcell, uint32_t *fb_id, uint32_t *fb_id1, int32_t *win,
                         uint32_t *wxy)
{
    const float (*v)[3] = s->v;
    float px = (float)x, py = (float)y;
    float w0 = orient(v[1][0], v[1][1], v[2][0], v[2][1], px, py);
    float w1 = orient(v[2][0], v[2][1], v[0][0], v[0][1], px, py);
    float w2 = orient(v[0][0], v[0][1], v[1][0], v[1][1], px, py);
    if (w0 >= 0.0f && w1 >= 0.0f && w2 >= 0.0f) {
        float shade = s->nz * s->a * (w0 + w1 + w2);
        float z = v[0][2] + s->a * (w1 * (v[1][2] - v[0][2]) + w2 * (v[2][2] - v[0][2]));
        if (z < *zcell) {
            *zcell = z;
            uint32_t px_cell = ORC_CELL(orc_default_shader(shade), s->rgb[0], s->rgb[1], s->rgb[2]);
            if (fb_id) *fb_id = px_cell;
            if (fb_id1) *fb_id1 = px_cell;
            if (win) *win = (int32_t)s->tri;
            if (wxy) *wxy = (uint32_t)x | ((uint32_t)y << 16);
        }
        (void)ctx;
        return 1;
    }
    return 0;
}

/* src/rasterizer.rs:48-93 draw_triangle, M = utransform*transform. */
void orc_draw_triangle(orc_ctx *ctx, const float v[9], const uint8_t rgb[3], const float M[16])
{
    orc_setup s;
    triangle_setup(ctx, v, rgb, M, ctx->next_tri++, &s);
    const uint64_t w = ctx->width;
    for (uint64_t y = s.y0; y < s.y1; ++y) {
        for (uint64_t x = s.x0; x < s.x1; ++x) {
            uint64_t id = y * w + x * 2;
            ctx->candidates++;
            ctx->fragments += (uint64_t)sample(ctx, &s, x, y, &ctx->z[id], &ctx->cells[id],
                                               &ctx->cells[id + 1],
                                               ctx->winner ? &ctx->winner[id] : NULL,
                                               ctx->winner_xy ? &ctx->winner_xy[id] : NULL);
        }
        if (ctx->image) ctx->cells[y * w + 1] = ORC_CELL('\n', 0, 0, 0);
    }
}

static void load_tri(const float *x, const float *y, const float *z, const uint32_t *idx,
                     uint32_t t, float v[9])
{
    for (int k = 0; k < 3; ++k) {
        uint64_t vi = idx ? idx[3 * (uint64_t)t + k] : 3 * (uint64_t)t + k;
        v[3 * k + 0] = x[vi];
        v[3 * k + 1] = y[vi];
        v[3 * k + 2] = z[vi];
    }
}

/* src/rasterizer.rs:39-46 draw_mesh. */
void orc_draw_mesh(orc_ctx *ctx, const float *x, const float *y, const float *z,
                   const uint32_t *idx, const uint8_t *rgb, uint32_t ntri, const float R[16])
{
    float M[16];
    orc_mat4_mul(ctx->U, R, M);
    for (uint32_t t = 0; t < ntri; ++t) {
        float v[9];
        load_tri(x, y, z, idx, t, v);
        orc_draw_triangle(ctx, v, rgb + 3 * (uint64_t)t, M);
    }
}

/* ---------------- banded (multi-threaded) form of the same sequence ---------------- */

typedef struct {
    orc_ctx *ctx;
    const orc_setup *setups;
    uint32_t ntri;
    uint64_t ra, rb;        /* owned target rows [ra, rb) */
    float ghost_z;          /* private copy of depth cell ra*w-1 (owned by the band above) */
    uint64_t fragments, candidates;
} band_job;

typedef struct {
    band_job *jobs;
    int njobs;
    int next;
    pthread_mutex_t mu;
} band_pool;

static void run_band(band_job *j)
{
    orc_ctx *ctx = j->ctx;
    const uint64_t w = ctx->width;
    const uint64_t lo = j->ra * w, hi = j->rb * w;
    const uint64_t ghost = lo - 1;          /* valid only when ra > 0 */
    for (uint32_t t = 0; t < j->ntri; ++t) {
        const orc_setup *s = &j->setups[t];
        if (s->y1 <= s->y0) continue;
        /* sample rows that can target rows [ra, rb): y in [ra-1, rb) */
        uint64_t ylo = j->ra > 0 ? j->ra - 1 : 0;
        uint64_t y_begin = s->y0 > ylo ? s->y0 : ylo;
        uint64_t y_end = s->y1 < j->rb ? s->y1 : j->rb;
        for (uint64_t y = y_begin; y < y_end; ++y) {
            for (uint64_t x = s->x0; x < s->x1; ++x) {
                uint64_t id = y * w + x * 2;
                if (id >= lo && id < hi) {
                    j->candidates++;
                    j->fragments += (uint64_t)sample(ctx, s, x, y, &ctx->z[id], &ctx->cells[id],
                                                     id + 1 < hi ? &ctx->cells[id + 1] : NULL,
                                                     ctx->winner ? &ctx->winner[id] : NULL,
                                                     ctx->winner_xy ? &ctx->winner_xy[id] : NULL);
                } else if (j->ra > 0 && id == ghost) {
                    /* the depth test of the cell above the band decides the write of
                       this band's first frame cell (its id+1 write) */
                    sample(ctx, s, x, y, &j->ghost_z, NULL, &ctx->cells[lo], NULL, NULL);
                }
            }
            if (ctx->image) {
                uint64_t c = y * w + 1;
                if (c >= lo && c < hi) ctx->cells[c] = ORC_CELL('\n', 0, 0, 0);
            }
        }
    }
}

static void *band_worker(void *arg)
{
    band_pool *p = (band_pool *)arg;
    for (;;) {
        pthread_mutex_lock(&p->mu);
        int i = p->next++;
        pthread_mutex_unlock(&p->mu);
        if (i >= p->njobs) break;
        run_band(&p->jobs[i]);
    }
    return NULL;
}

void orc_draw_mesh_banded(orc_ctx *ctx, const float *x, const float *y, const float *z,
                          const uint32_t *idx, const uint8_t *rgb, uint32_t ntri,
                          const float R[16], int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    float M[16];
    orc_mat4_mul(ctx->U, R, M);
    orc_setup *setups = (orc_setup *)malloc(sizeof(orc_setup) * (ntri ? ntri : 1));
    for (uint32_t t = 0; t < ntri; ++t) {
        float v[9];
        load_tri(x, y, z, idx, t, v);
        triangle_setup(ctx, v, rgb + 3 * (uint64_t)t, M, ctx->next_tri + t, &setups[t]);
    }
    ctx->next_tri += ntri;
    /* rows in bands of a few rows each, handed out dynamically */
    uint64_t h = ctx->height;
    uint64_t rows_per = h / ((uint64_t)nthreads * 8);
    if (rows_per < 1) rows_per = 1;
    int njobs = (int)((h + rows_per - 1) / rows_per);
    band_job *jobs = (band_job *)calloc((size_t)(njobs ? njobs : 1), sizeof(band_job));
    const uint64_t w = ctx->width;
    for (int i = 0; i < njobs; ++i) {
        jobs[i].ctx = ctx;
        jobs[i].setups = setups;
        jobs[i].ntri = ntri;
        jobs[i].ra = (uint64_t)i * rows_per;
        jobs[i].rb = jobs[i].ra + rows_per < h ? jobs[i].ra + rows_per : h;
        /* read before any band writes: the depth cell above the band as it stands now */
        jobs[i].ghost_z = jobs[i].ra > 0 ? ctx->z[jobs[i].ra * w - 1] : ORC_FLT_MAX;
    }
    band_pool pool = { jobs, njobs, 0, PTHREAD_MUTEX_INITIALIZER };
    int nt = nthreads < njobs ? nthreads : njobs;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)(nt > 0 ? nt : 1));
    for (int i = 0; i < nt; ++i) pthread_create(&th[i], NULL, band_worker, &pool);
    for (int i = 0; i < nt; ++i) pthread_join(th[i], NULL);
    for (int i = 0; i < njobs; ++i) {
        ctx->fragments += jobs[i].fragments;
        ctx->candidates += jobs[i].candidates;
    }
    free(th);
    free(jobs);
    free(setups);
}

/* ---------------- Context::flush (src/context.rs:50-92) ---------------- */

static uint64_t put_bytes(char *out, uint64_t at, const char *s, uint64_t n)
{
    if (out) memcpy(out + at, s, n);
    return n;
}

uint64_t orc_flush(const uint32_t *cells, uint64_t ncells, int image, int format, char *out)
{
    uint64_t n = 0;
    char buf[64];
    if (!image) n += put_bytes(out, n, "\x1b[1;1H", 6);          /* stdout.queue(cursor::MoveTo(0, 0)) */
    for (uint64_t i = 0; i < ncells; ++i) {
        const unsigned ch = cells[i] & 255u, r = (cells[i] >> 8) & 255u, g = (cells[i] >> 16) & 255u,
                       b = cells[i] >> 24;
        int k;
        if (format == 0) {
            buf[0] = (char)ch;
            k = 1;
        } else if (format == 1) {
            k = snprintf(buf, sizeof buf, "\x1b[48;2;25;25;25m\x1b[38;2;%u;%u;%um%c\x1b[0m", r, g, b, (char)ch);
        } else {
            k = snprintf(buf, sizeof buf, "<span style=\"color:rgb(%u,%u,%u)\">%c", r, g, b, (char)ch);
        }
        n += put_bytes(out, n, buf, (uint64_t)k);
    }
    if (format == 0) n += put_bytes(out, n, "\n", 1);            /* println!("{}", frame) */
    return n;
}

