// sloth_api.cpp -- the C ABI (include/sloth_gpu.h): contexts, meshes and the draw path.
//
// Host-side restatement of the reference's per-frame driver around the hot path:
// Context::blank/update/clear (src/context.rs:22-45, 93-141), draw_mesh
// (src/rasterizer.rs:39-46) and the buffer reads that Context::flush prints.  All device
// memory is owned here; all work is ordered on the context's stream (two kernels of a
// draw run on helper streams forked from it and joined back).  There is no CPU fallback:
// if CUDA or the kernels are unavailable every call fails with SLOTH_ERR_CUDA.
//
// Host float math below must be compiled with -ffp-contract=off (see build.py).
#include "sloth_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "sloth_internal.cuh"
#include "sloth_kernels.h"
#include "flush_kernels.h"

using namespace sloth;

namespace {

struct EventPair {
    cudaEvent_t a, b;
};
struct KernelClock {
    double ms = 0.0;
    uint64_t launches = 0;
    std::vector<EventPair> pending;
};

}  // namespace

// batch_api.cu: frees a batch's device memory and cuts it from its context.
void sloth_batch_detach(sloth_batch *b);

struct sloth_mesh {
    sloth_ctx *ctx = nullptr;
    int device = 0;
    float *x = nullptr, *y = nullptr, *z = nullptr;
    uint32_t *idx = nullptr;
    uint8_t *rgb = nullptr;
    uint32_t nvert = 0, ntri = 0;
    float bbox_max[3] = {0, 0, 0};
    uint32_t *order = nullptr, *oidx = nullptr;   // setup's order of an indexed mesh (spatial_order)
};

struct sloth_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;

    // requested viewport (Context.width/height/image) and utransform
    uint32_t req_w = 0, req_h = 0;
    int req_image = 0;
    float U[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

    // allocated frame state
    bool have_frame = false;
    FrameGeom g{};
    FrameBuffers fb{};
    size_t records_cap = 0;
    BinBuffers bb{};
    uint32_t ntiles_cap = 0;
    size_t large_cap = 0;
    size_t fill_cap = 0;
    float4 *tv = nullptr;
    size_t tv_cap = 0;
    uint32_t *h_total = nullptr;   // pinned
    cudaEvent_t total_ev = nullptr;   // h_total has arrived
    uint32_t *d_max = nullptr;     // largest entry total of any draw (the scan's atomicMax)
    uint32_t *h_max = nullptr;     // pinned copy of d_max
    cudaEvent_t max_ev = nullptr;  // h_max has arrived
    bool max_pending = false;      // a copy of d_max is on its way
    unsigned long long *h_frags = nullptr;   // pinned
    uint32_t *h_error = nullptr;   // pinned copy of fb.error
    uint32_t tri_base = 0;
    bool dirty = true;
    bool reset_pending = false;    // a clear's resets, folded into the next launch that needs them
    cudaStream_t side = nullptr;   // the entry-count copy, off the draw's stream
    cudaEvent_t scan_ev = nullptr;
    cudaStream_t nl_stream = nullptr;   // the newline fold, beside the binning kernels
    cudaStream_t aux = nullptr;         // the large-triangle fill, beside the small one
    cudaEvent_t fill_ev = nullptr, aux_ev = nullptr;
    cudaEvent_t setup_ev = nullptr, nl_ev = nullptr;
    bool nl_pending = false;            // a newline fold not yet joined into the ctx stream

    // instrumentation and options
    int depth_cull = 1;
    int tile_shape = 0;
    int direct_max = 0;            // SLOTH_OPTION_DIRECT_SAMPLES (applied at the next clear)
    int tpb = kDefaultTrianglesPerBlock;   // SLOTH_OPTION_TRIANGLES_PER_BLOCK
    bool keys_current = false;     // every tile's keys cleared for the current generation
    bool timing = false;
    std::map<std::string, KernelClock> clocks;
    uint64_t launches = 0;

    FlushScratch flush;

    // handles made on this context: released or detached when it is destroyed
    std::vector<sloth_mesh *> meshes;
    std::vector<sloth_batch *> batches;
};

// ---------------------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------------------
static sloth_status fail(sloth_ctx *ctx, sloth_status st, const char *fmt, ...)
{
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return st;
}

#define CU(ctx, call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return fail((ctx), e_ == cudaErrorMemoryAllocation ? SLOTH_ERR_OUT_OF_MEMORY \
                                                               : SLOTH_ERR_CUDA,        \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                \
    } while (0)

template <class T>
static cudaError_t dalloc(T **p, size_t n)
{
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T));
}

template <class T>
static void dfree(T *&p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

// Time one launch on stream s (default: the ctx stream) when timing is enabled.
template <class F>
static cudaError_t timed(sloth_ctx *ctx, const char *name, F &&launch, cudaStream_t s = nullptr)
{
    if (!s) s = ctx->stream;
    if (!ctx->timing) {
        cudaError_t e = launch();
        if (e == cudaSuccess) ctx->launches++;
        return e;
    }
    EventPair ev;
    cudaEventCreate(&ev.a);
    cudaEventCreate(&ev.b);
    cudaEventRecord(ev.a, s);
    cudaError_t e = launch();
    cudaEventRecord(ev.b, s);
    if (e == cudaSuccess) {
        ctx->launches++;
        ctx->clocks[name].pending.push_back(ev);
    } else {
        cudaEventDestroy(ev.a);
        cudaEventDestroy(ev.b);
    }
    return e;
}

// Waits for the context's helper streams (newline fold, entry-count copy) before device
// memory they may read is released.
static void quiesce_helpers(sloth_ctx *ctx)
{
    if (ctx->nl_stream) cudaStreamSynchronize(ctx->nl_stream);
    if (ctx->aux) cudaStreamSynchronize(ctx->aux);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    ctx->nl_pending = false;
}

static void free_frame(sloth_ctx *ctx)
{
    quiesce_helpers(ctx);
    dfree(ctx->fb.keys);
    dfree(ctx->fb.tile_gen);
    dfree(ctx->fb.nltree);
    dfree(ctx->fb.z_out);
    dfree(ctx->fb.cells_out);
    dfree(ctx->fb.winner_out);
    dfree(ctx->fb.fragments);
    dfree(ctx->bb.tile_count);
    dfree(ctx->bb.tile_offset);
    dfree(ctx->bb.tile_cursor);
    dfree(ctx->bb.slice_offset);
    ctx->have_frame = false;
    ctx->ntiles_cap = 0;
}

// (Re)allocate the per-frame buffers for the requested viewport.
static sloth_status alloc_frame(sloth_ctx *ctx)
{
    free_frame(ctx);
    FrameGeom g{};
    g.w = (int32_t)ctx->req_w;
    g.h = (int32_t)ctx->req_h;
    g.image = ctx->req_image ? 1 : 0;
    g.tw = kTileShapes[ctx->tile_shape][0];
    g.th = kTileShapes[ctx->tile_shape][1];
    g.ntx = (g.w + g.tw - 1) / g.tw;
    g.nty = (g.h + g.th - 1) / g.th;
    g.pitch = g.ntx * g.tw;
    g.nl_size = 1;
    while (g.nl_size < g.h) g.nl_size <<= 1;
    const size_t ntiles = (size_t)g.ntx * g.nty;
    const size_t nz = (size_t)g.w * g.h;
    const size_t ncells = g.image ? nz + g.h : nz;
    CU(ctx, dalloc(&ctx->fb.keys, (size_t)g.pitch * g.nty * g.th));
    CU(ctx, dalloc(&ctx->fb.tile_gen, ntiles));
    CU(ctx, cudaMemsetAsync(ctx->fb.tile_gen, 0, ntiles * sizeof(uint32_t), ctx->stream));
    CU(ctx, dalloc(&ctx->fb.nltree, 2 * (size_t)g.nl_size));
    CU(ctx, dalloc(&ctx->fb.z_out, nz));
    CU(ctx, dalloc(&ctx->fb.cells_out, ncells));
    CU(ctx, dalloc(&ctx->fb.winner_out, nz));
    CU(ctx, dalloc(&ctx->fb.fragments, 1));
    CU(ctx, dalloc(&ctx->bb.tile_count, ntiles));
    CU(ctx, dalloc(&ctx->bb.tile_offset, ntiles + 1));
    CU(ctx, dalloc(&ctx->bb.tile_cursor, ntiles));
    CU(ctx, dalloc(&ctx->bb.slice_offset, ntiles + kSliceExtra));
    ctx->ntiles_cap = (uint32_t)ntiles;
    ctx->fb.gen = 0;
    ctx->g = g;
    ctx->have_frame = true;
    return SLOTH_OK;
}

static sloth_status ensure_records(sloth_ctx *ctx, size_t need)
{
    if (need <= ctx->records_cap) return SLOTH_OK;
    size_t cap = ctx->records_cap ? ctx->records_cap : 1024;
    while (cap < need) cap *= 2;
    TriRecord *n = nullptr;
    uint32_t *rows = nullptr;
    CU(ctx, dalloc(&n, cap));
    CU(ctx, dalloc(&rows, cap));   // read only by the newline fold of the draw that wrote them
    if (ctx->fb.records && ctx->tri_base)
        CU(ctx, cudaMemcpyAsync(n, ctx->fb.records, (size_t)ctx->tri_base * sizeof(TriRecord),
                                cudaMemcpyDeviceToDevice, ctx->stream));
    CU(ctx, cudaStreamSynchronize(ctx->stream));
    quiesce_helpers(ctx);
    dfree(ctx->fb.records);
    dfree(ctx->fb.rows);
    ctx->fb.records = n;
    ctx->fb.rows = rows;
    ctx->records_cap = cap;
    return SLOTH_OK;
}

template <class T>
static sloth_status ensure_scratch(sloth_ctx *ctx, T **p, size_t *cap, size_t need)
{
    if (need <= *cap && *p) return SLOTH_OK;
    size_t c = *cap ? *cap : 1024;
    while (c < need) c *= 2;
    CU(ctx, cudaStreamSynchronize(ctx->stream));
    quiesce_helpers(ctx);
    dfree(*p);
    CU(ctx, dalloc(p, c));
    *cap = c;
    return SLOTH_OK;
}

// A clear's resets (error word, fragments, newline tree) wait for the next launch that
// reads them; a draw adds its own (tile counts, large-queue counters) to the same launch.
static sloth_status apply_resets(sloth_ctx *ctx, bool draw)
{
    if (!ctx->reset_pending && !draw) return SLOTH_OK;
    const bool frame = ctx->reset_pending;
    // a draw that folds small triangles straight into the global keys needs every tile's
    // keys valid for this generation: cleared once per frame, the tiles made current
    const bool tiles = draw && ctx->g.direct_max > 0 && !ctx->keys_current;
    if (tiles)
        CU(ctx, launch_clear_keys(ctx->fb.keys, (uint64_t)ctx->g.pitch * ctx->g.nty * ctx->g.th, ctx->g.tw,
                                  !(ctx->g.w & 1), ctx->stream));
    CU(ctx, timed(ctx, "reset", [&] {
           return launch_frame_reset(ctx->fb, ctx->bb, 2u * (uint32_t)ctx->g.nl_size,
                                     (uint32_t)(ctx->g.ntx * ctx->g.nty), frame, draw, tiles, ctx->stream);
       }));
    ctx->reset_pending = false;
    if (tiles) ctx->keys_current = true;
    return SLOTH_OK;
}

// The device error word travels with the next synchronising call's copies.
static sloth_status queue_error_copy(sloth_ctx *ctx)
{
    if (ctx->have_frame) {
        sloth_status st0 = apply_resets(ctx, false);
        if (st0 != SLOTH_OK) return st0;
    }
    CU(ctx, cudaMemcpyAsync(ctx->h_error, ctx->fb.error, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    return SLOTH_OK;
}

// After a stream synchronisation that followed queue_error_copy.
static sloth_status report_device_error(sloth_ctx *ctx)
{
    if (*ctx->h_error)
        return fail(ctx, SLOTH_ERR_DEVICE_FAULT, "a raster block gave up waiting for its tile copy (code %u)",
                    *ctx->h_error);
    return SLOTH_OK;
}

// The ctx stream waits for the last newline fold (before a resolve or the next draw).
static sloth_status join_newline(sloth_ctx *ctx)
{
    if (!ctx->nl_pending) return SLOTH_OK;
    CU(ctx, cudaStreamWaitEvent(ctx->stream, ctx->nl_ev, 0));
    ctx->nl_pending = false;
    return SLOTH_OK;
}

static sloth_status resolve_pending(sloth_ctx *ctx)
{
    if (!ctx->have_frame)
        return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "the context has no frame: call sloth_ctx_clear first");
    sloth_status st0 = apply_resets(ctx, false);
    if (st0 != SLOTH_OK) return st0;
    if ((st0 = join_newline(ctx)) != SLOTH_OK) return st0;
    if (!ctx->dirty) return SLOTH_OK;
    CU(ctx, timed(ctx, "resolve", [&] { return launch_resolve(ctx->g, ctx->fb, ctx->stream); }));
    ctx->dirty = false;
    return SLOTH_OK;
}

// ---------------------------------------------------------------------------------------
// accessors for the batch API (batch_api.cu)
// ---------------------------------------------------------------------------------------
sloth_status sloth_ctx_fail(sloth_ctx *ctx, sloth_status st, const char *msg) { return fail(ctx, st, "%s", msg); }
void sloth_ctx_register_batch(sloth_ctx *ctx, sloth_batch *b) { ctx->batches.push_back(b); }
void sloth_ctx_unregister_batch(sloth_ctx *ctx, sloth_batch *b)
{
    auto &v = ctx->batches;
    v.erase(std::remove(v.begin(), v.end(), b), v.end());
}
int sloth_ctx_device(const sloth_ctx *ctx) { return ctx->device; }
cudaStream_t sloth_ctx_stream(const sloth_ctx *ctx) { return ctx->stream; }
int sloth_ctx_depth_cull(const sloth_ctx *ctx) { return ctx->depth_cull; }
int sloth_ctx_direct_samples(const sloth_ctx *ctx) { return ctx->direct_max; }
struct MeshView {
    const float *x, *y, *z;
    const uint32_t *idx;
    const uint8_t *rgb;
    uint32_t nvert, ntri;
    int device;
    const uint32_t *order, *oidx;   // setup's order of an indexed mesh (MeshDev), or null
};
MeshView sloth_mesh_view(const sloth_mesh *m)
{
    return MeshView{m->x, m->y, m->z, m->idx, m->rgb, m->nvert, m->ntri, m->device, m->order, m->oidx};
}

// ---------------------------------------------------------------------------------------
// host math (restated from the reference and nalgebra 0.22.1; -ffp-contract=off)
// ---------------------------------------------------------------------------------------
extern "C" {

const char *sloth_version(void) { return "sloth-gb300 0.1 (sm_103a)"; }

void sloth_shader_thresholds(float thresholds[9], char chars[10])
{
    static const float t[9] = {0.20f, 0.30f, 0.40f, 0.50f, 0.60f, 0.70f, 0.80f, 0.90f, 1.0f};
    static const char c[10] = {'.', ':', '-', '=', '+', '*', '#', '%', '@', ' '};
    if (thresholds) memcpy(thresholds, t, sizeof t);
    if (chars) memcpy(chars, c, sizeof c);
}

// src/rasterizer.rs:5-27
char sloth_default_shader(float shade)
{
    if (shade <= 0.20f) return '.';
    if (shade <= 0.30f) return ':';
    if (shade <= 0.40f) return '-';
    if (shade <= 0.50f) return '=';
    if (shade <= 0.60f) return '+';
    if (shade <= 0.70f) return '*';
    if (shade <= 0.80f) return '#';
    if (shade <= 0.90f) return '%';
    if (shade <= 1.0f) return '@';
    return ' ';
}

// nalgebra Rotation3::from_euler_angles (ZYX) + to_homogeneous, src/main.rs:76-77.
void sloth_euler_rotation(float roll, float pitch, float yaw, float out[16])
{
    const float sr = std::sin(roll), cr = std::cos(roll);
    const float sp = std::sin(pitch), cp = std::cos(pitch);
    const float sy = std::sin(yaw), cy = std::cos(yaw);
    const float m[16] = {
        cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr, 0.0f,
        sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr, 0.0f,
        -sp,     cp * sr,                cp * cr,                0.0f,
        0.0f,    0.0f,                   0.0f,                   1.0f,
    };
    memcpy(out, m, sizeof m);
}

// nalgebra gemm -> gemv: column by column, first product then + each later product.
void sloth_mat4_mul(const float a[16], const float b[16], float out[16])
{
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float acc = a[i * 4 + 0] * b[0 * 4 + j];
            for (int k = 1; k < 4; ++k) acc = a[i * 4 + k] * b[k * 4 + j] + acc;
            r[i * 4 + j] = acc;
        }
    memcpy(out, r, sizeof r);
}

// src/context.rs:106-113
float sloth_scene_extent(const float *bbox_max, uint32_t nmesh)
{
    float s = 0.0f;
    for (uint32_t m = 0; m < nmesh; ++m)
        for (int k = 0; k < 3; ++k) s = std::fmax(s, bbox_max[3 * m + k]);
    return s;
}

// src/context.rs:114-133
void sloth_viewport_transform(uint16_t width, uint16_t height, float extent, float out[16])
{
    const float fw = (float)width, fh = (float)height;
    const float scale = std::fmin(fh, fw / 2.0f) / extent / 2.0f;
    const float t[16] = {scale, 0.0f,   0.0f,  fw / 4.0f, 0.0f, -scale, 0.0f, fh / 2.0f,
                         0.0f,  0.0f,   scale, 0.0f,      0.0f, 0.0f,   0.0f, 1.0f};
    memcpy(out, t, sizeof t);
}

// ---------------------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------------------
sloth_status sloth_ctx_create(sloth_ctx **out, int device, void *stream)
{
    if (!out) return SLOTH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SLOTH_ERR_CUDA;
    if (device < 0 || device >= ndev) return SLOTH_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return SLOTH_ERR_CUDA;
    sloth_ctx *ctx = new sloth_ctx();
    ctx->device = device;
    if (stream) {
        ctx->stream = static_cast<cudaStream_t>(stream);
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete ctx;
            return SLOTH_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    if (cudaMallocHost(&ctx->h_total, sizeof(uint32_t)) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->total_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->scan_ev, cudaEventDisableTiming) != cudaSuccess ||
        prepare_setup_kernels() != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->nl_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->fill_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->aux_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->setup_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->nl_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost(&ctx->h_frags, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_error, sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&ctx->fb.error, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(ctx->fb.error, 0, sizeof(uint32_t)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_max, sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&ctx->d_max, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(ctx->d_max, 0, sizeof(uint32_t)) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->max_ev, cudaEventDisableTiming) != cudaSuccess) {
        if (ctx->h_total) cudaFreeHost(ctx->h_total);
        if (ctx->total_ev) cudaEventDestroy(ctx->total_ev);
        if (ctx->scan_ev) cudaEventDestroy(ctx->scan_ev);
        if (ctx->side) cudaStreamDestroy(ctx->side);
        if (ctx->nl_stream) cudaStreamDestroy(ctx->nl_stream);
        if (ctx->aux) cudaStreamDestroy(ctx->aux);
        if (ctx->setup_ev) cudaEventDestroy(ctx->setup_ev);
        if (ctx->nl_ev) cudaEventDestroy(ctx->nl_ev);
        if (ctx->fill_ev) cudaEventDestroy(ctx->fill_ev);
        if (ctx->aux_ev) cudaEventDestroy(ctx->aux_ev);
        if (ctx->h_frags) cudaFreeHost(ctx->h_frags);
        if (ctx->h_error) cudaFreeHost(ctx->h_error);
        if (ctx->fb.error) cudaFree(ctx->fb.error);
        if (ctx->h_max) cudaFreeHost(ctx->h_max);
        if (ctx->d_max) cudaFree(ctx->d_max);
        if (ctx->max_ev) cudaEventDestroy(ctx->max_ev);
        if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return SLOTH_ERR_OUT_OF_MEMORY;
    }
    *ctx->h_error = 0;
    *ctx->h_max = 0;
    ctx->bb.max_total = ctx->d_max;
    *out = ctx;
    return SLOTH_OK;
}

void sloth_ctx_destroy(sloth_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    quiesce_helpers(ctx);
    // batches lose their device memory and meshes their context; destroying either
    // afterwards only frees what is left
    for (sloth_batch *b : ctx->batches) sloth_batch_detach(b);
    for (sloth_mesh *m : ctx->meshes) m->ctx = nullptr;
    for (auto &kv : ctx->clocks)
        for (auto &ev : kv.second.pending) {
            cudaEventDestroy(ev.a);
            cudaEventDestroy(ev.b);
        }
    free_frame(ctx);
    dfree(ctx->fb.records);
    dfree(ctx->fb.rows);
    dfree(ctx->bb.entries);
    dfree(ctx->bb.large_queue);
    dfree(ctx->bb.fill_list);
    dfree(ctx->bb.large_count);
    dfree(ctx->bb.items);
    dfree(ctx->tv);
    if (ctx->h_total) cudaFreeHost(ctx->h_total);
    if (ctx->total_ev) cudaEventDestroy(ctx->total_ev);
    if (ctx->scan_ev) cudaEventDestroy(ctx->scan_ev);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->nl_stream) cudaStreamDestroy(ctx->nl_stream);
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    if (ctx->setup_ev) cudaEventDestroy(ctx->setup_ev);
    if (ctx->nl_ev) cudaEventDestroy(ctx->nl_ev);
    if (ctx->fill_ev) cudaEventDestroy(ctx->fill_ev);
    if (ctx->aux_ev) cudaEventDestroy(ctx->aux_ev);
    if (ctx->h_frags) cudaFreeHost(ctx->h_frags);
    if (ctx->h_error) cudaFreeHost(ctx->h_error);
    dfree(ctx->fb.error);
    if (ctx->h_max) cudaFreeHost(ctx->h_max);
    dfree(ctx->d_max);
    if (ctx->max_ev) cudaEventDestroy(ctx->max_ev);
    flush_release(ctx->flush);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char *sloth_ctx_last_error(const sloth_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

sloth_status sloth_ctx_set_viewport(sloth_ctx *ctx, uint32_t width, uint32_t height, int image)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    if (width < 1 || height < 1 || width > SLOTH_MAX_DIM || height > SLOTH_MAX_DIM)
        return fail(ctx, SLOTH_ERR_LIMIT, "viewport %ux%u outside 1..%u", width, height, SLOTH_MAX_DIM);
    ctx->req_w = width;
    ctx->req_h = height;
    ctx->req_image = image ? 1 : 0;
    return SLOTH_OK;
}

sloth_status sloth_ctx_set_utransform(sloth_ctx *ctx, const float u[16])
{
    if (!ctx || !u) return SLOTH_ERR_INVALID_ARGUMENT;
    memcpy(ctx->U, u, sizeof ctx->U);
    return SLOTH_OK;
}

sloth_status sloth_ctx_update(sloth_ctx *ctx, const sloth_mesh *const *meshes, uint32_t nmesh)
{
    if (!ctx || (nmesh && !meshes)) return SLOTH_ERR_INVALID_ARGUMENT;
    std::vector<float> bb(3 * (size_t)nmesh);
    for (uint32_t i = 0; i < nmesh; ++i) {
        if (!meshes[i]) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "mesh %u is NULL", i);
        memcpy(&bb[3 * (size_t)i], meshes[i]->bbox_max, 3 * sizeof(float));
    }
    const float ext = sloth_scene_extent(bb.data(), nmesh);
    sloth_viewport_transform((uint16_t)ctx->req_w, (uint16_t)ctx->req_h, ext, ctx->U);
    return SLOTH_OK;
}

sloth_status sloth_ctx_clear(sloth_ctx *ctx)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    if (ctx->req_w == 0 || ctx->req_h == 0)
        return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "no viewport: call sloth_ctx_set_viewport first");
    CU(ctx, cudaSetDevice(ctx->device));
    if (!ctx->have_frame || ctx->g.w != (int32_t)ctx->req_w || ctx->g.h != (int32_t)ctx->req_h ||
        ctx->g.image != ctx->req_image || ctx->g.tw != kTileShapes[ctx->tile_shape][0] ||
        ctx->g.th != kTileShapes[ctx->tile_shape][1]) {
        sloth_status st = alloc_frame(ctx);
        if (st != SLOTH_OK) return st;
    }
    // A new frame starts without a device error, fragments or newlines (reset by the next
    // launch that needs them).
    ctx->reset_pending = true;
    // A new generation invalidates every tile's keys without touching them.
    ctx->fb.gen++;
    if (ctx->fb.gen == 0) {
        CU(ctx, cudaMemsetAsync(ctx->fb.tile_gen, 0, ctx->ntiles_cap * sizeof(uint32_t), ctx->stream));
        ctx->fb.gen = 1;
    }
    ctx->tri_base = 0;
    ctx->dirty = true;
    ctx->g.direct_max = ctx->direct_max;
    ctx->keys_current = false;
    return SLOTH_OK;
}

sloth_status sloth_ctx_sizes(const sloth_ctx *ctx, uint64_t *frame_cells, uint64_t *depth_cells)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    const uint64_t nz = (uint64_t)ctx->req_w * ctx->req_h;
    if (frame_cells) *frame_cells = ctx->req_image ? nz + ctx->req_h : nz;
    if (depth_cells) *depth_cells = nz;
    return SLOTH_OK;
}

sloth_status sloth_ctx_read(sloth_ctx *ctx, uint32_t *cells, float *z, int32_t *winner)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    CU(ctx, cudaSetDevice(ctx->device));
    sloth_status st = resolve_pending(ctx);
    if (st != SLOTH_OK) return st;
    const size_t nz = (size_t)ctx->g.w * ctx->g.h;
    const size_t ncells = ctx->g.image ? nz + ctx->g.h : nz;
    if (cells)
        CU(ctx, cudaMemcpyAsync(cells, ctx->fb.cells_out, ncells * sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, ctx->stream));
    if (z)
        CU(ctx, cudaMemcpyAsync(z, ctx->fb.z_out, nz * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (winner)
        CU(ctx, cudaMemcpyAsync(winner, ctx->fb.winner_out, nz * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = queue_error_copy(ctx)) != SLOTH_OK) return st;
    CU(ctx, cudaStreamSynchronize(ctx->stream));
    return report_device_error(ctx);
}

static sloth_status ctx_flush(sloth_ctx *ctx, int format, uint64_t *bytes)
{
    if (format < SLOTH_FLUSH_PLAIN || format > SLOTH_FLUSH_HTML)
        return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "unknown flush format %d", format);
    CU(ctx, cudaSetDevice(ctx->device));
    sloth_status st = resolve_pending(ctx);
    if (st != SLOTH_OK) return st;
    const uint64_t nz = (uint64_t)ctx->g.w * ctx->g.h;
    const uint64_t ncells = ctx->g.image ? nz + ctx->g.h : nz;
    if ((st = queue_error_copy(ctx)) != SLOTH_OK) return st;
    CU(ctx, timed(ctx, "flush", [&] {
        return flush_run(ctx->flush, ctx->fb.cells_out, ncells, ctx->g.image, format, ctx->stream, bytes);
    }));
    return report_device_error(ctx);
}

sloth_status sloth_ctx_flush(sloth_ctx *ctx, int format, char *out, uint64_t capacity, uint64_t *bytes)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    if (!bytes) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "bytes is NULL");
    sloth_status st = ctx_flush(ctx, format, bytes);
    if (st != SLOTH_OK || !out) return st;
    if (capacity < *bytes) return fail(ctx, SLOTH_ERR_LIMIT, "flush needs %llu bytes", (unsigned long long)*bytes);
    CU(ctx, cudaMemcpyAsync(out, ctx->flush.out, *bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CU(ctx, cudaStreamSynchronize(ctx->stream));
    return SLOTH_OK;
}

sloth_status sloth_ctx_flush_device(sloth_ctx *ctx, int format, const char **device_bytes, uint64_t *bytes)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    if (!bytes || !device_bytes) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "bytes/device_bytes is NULL");
    sloth_status st = ctx_flush(ctx, format, bytes);
    if (st != SLOTH_OK) return st;
    *device_bytes = ctx->flush.out;
    return SLOTH_OK;
}

sloth_status sloth_ctx_read_async(sloth_ctx *ctx, uint32_t *cells, float *z, int32_t *winner)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    CU(ctx, cudaSetDevice(ctx->device));
    sloth_status st = resolve_pending(ctx);
    if (st != SLOTH_OK) return st;
    const size_t nz = (size_t)ctx->g.w * ctx->g.h;
    const size_t ncells = ctx->g.image ? nz + ctx->g.h : nz;
    if (cells)
        CU(ctx, cudaMemcpyAsync(cells, ctx->fb.cells_out, ncells * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                ctx->stream));
    if (z) CU(ctx, cudaMemcpyAsync(z, ctx->fb.z_out, nz * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (winner)
        CU(ctx, cudaMemcpyAsync(winner, ctx->fb.winner_out, nz * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                ctx->stream));
    return queue_error_copy(ctx);
}

sloth_status sloth_ctx_synchronize(sloth_ctx *ctx)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    CU(ctx, cudaSetDevice(ctx->device));
    sloth_status st = queue_error_copy(ctx);
    if (st != SLOTH_OK) return st;
    if ((st = join_newline(ctx)) != SLOTH_OK) return st;   // every kernel of the context is done
    CU(ctx, cudaStreamSynchronize(ctx->stream));
    return report_device_error(ctx);
}

sloth_status sloth_ctx_device_buffers(sloth_ctx *ctx, const uint32_t **cells, const float **z)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    CU(ctx, cudaSetDevice(ctx->device));
    sloth_status st = resolve_pending(ctx);
    if (st != SLOTH_OK) return st;
    if (cells) *cells = ctx->fb.cells_out;
    if (z) *z = ctx->fb.z_out;
    return SLOTH_OK;
}

sloth_status sloth_ctx_fragments(sloth_ctx *ctx, uint64_t *fragments)
{
    if (!ctx || !fragments) return SLOTH_ERR_INVALID_ARGUMENT;
    if (!ctx->have_frame) {
        *fragments = 0;
        return SLOTH_OK;
    }
    CU(ctx, cudaSetDevice(ctx->device));
    sloth_status st = apply_resets(ctx, false);
    if (st != SLOTH_OK) return st;
    CU(ctx, cudaMemcpyAsync(ctx->h_frags, ctx->fb.fragments, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, ctx->stream));
    st = queue_error_copy(ctx);
    if (st != SLOTH_OK) return st;
    CU(ctx, cudaStreamSynchronize(ctx->stream));
    *fragments = *ctx->h_frags;
    return report_device_error(ctx);
}

// ---------------------------------------------------------------------------------------
// meshes
// ---------------------------------------------------------------------------------------
// Setup's order of an indexed mesh's triangles: ascending Morton code (10 bits an axis,
// interleaved x, y, z from the lowest bit) of the centroid's place in the box of the
// finite centroids, ties in index order; a triangle with a non-finite centroid takes code
// 0.  Triangles next to each other in this order lie close together in space, so the
// triangles one warp or block sets up land on nearby cells and tiles in any view, and
// their depth-key reductions and tile counts share cache lines and atomics.  The results
// do not depend on the order (every output is indexed by the triangle), only the speed.
static void spatial_order(const float *x, const float *y, const float *z, const uint32_t *idx, uint32_t ntri,
                          std::vector<uint32_t> &order)
{
    const float *v[3] = {x, y, z};
    std::vector<float> c(3 * (size_t)ntri);
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t t = 0; t < ntri; ++t) {
        const uint32_t *i = idx + 3 * (size_t)t;
        for (int a = 0; a < 3; ++a) {
            const float s = v[a][i[0]] + v[a][i[1]] + v[a][i[2]];
            c[3 * (size_t)t + a] = s;
            if (std::isfinite(s)) {
                lo[a] = std::fmin(lo[a], s);
                hi[a] = std::fmax(hi[a], s);
            }
        }
    }
    std::vector<uint32_t> code(ntri);
    for (uint32_t t = 0; t < ntri; ++t) {
        uint32_t q[3];
        bool finite = true;
        for (int a = 0; a < 3; ++a) {
            const float s = c[3 * (size_t)t + a];
            finite = finite && std::isfinite(s);
            const double f = hi[a] > lo[a] ? ((double)s - lo[a]) / ((double)hi[a] - lo[a]) : 0.0;
            q[a] = f <= 0.0 ? 0u : f >= 1.0 ? 1023u : (uint32_t)(f * 1024.0);
        }
        uint32_t m = 0;
        if (finite)
            for (int b = 0; b < 10; ++b)
                for (int a = 0; a < 3; ++a) m |= ((q[a] >> b) & 1u) << (3 * b + a);
        code[t] = m;
    }
    // stable least-significant-digit radix sort of the 30-bit codes, two digits of 15 bits
    std::vector<uint32_t> src(ntri), cnt(1u << 15);
    for (uint32_t t = 0; t < ntri; ++t) src[t] = t;
    order.assign(ntri, 0u);
    for (int shift = 0; shift < 30; shift += 15) {
        std::fill(cnt.begin(), cnt.end(), 0u);
        for (uint32_t t : src) ++cnt[(code[t] >> shift) & 0x7fffu];
        uint32_t run = 0;
        for (uint32_t &k : cnt) {
            const uint32_t n = k;
            k = run;
            run += n;
        }
        for (uint32_t t : src) order[cnt[(code[t] >> shift) & 0x7fffu]++] = t;
        src.swap(order);
    }
    order.swap(src);
}

sloth_status sloth_spatial_order(const float *x, const float *y, const float *z, uint32_t nvert, const uint32_t *idx,
                                 uint32_t ntri, uint32_t *order)
{
    if (ntri && (!x || !y || !z || !idx || !order)) return SLOTH_ERR_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < 3ull * ntri; ++i)
        if (idx[i] >= nvert) return SLOTH_ERR_INVALID_ARGUMENT;
    try {
        std::vector<uint32_t> ord;
        spatial_order(x, y, z, idx, ntri, ord);
        std::copy(ord.begin(), ord.end(), order);
    } catch (const std::bad_alloc &) {
        return SLOTH_ERR_OUT_OF_MEMORY;
    }
    return SLOTH_OK;
}

sloth_status sloth_mesh_create(sloth_ctx *ctx, const float *x, const float *y, const float *z,
                               uint32_t nvert, const uint32_t *idx, uint32_t ntri,
                               const uint8_t *rgb, const float *bbox_max, sloth_mesh **out)
{
    if (!ctx || !out) return SLOTH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (nvert && (!x || !y || !z)) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "vertex arrays are NULL");
    if (ntri && !rgb) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "rgb is NULL");
    if (!idx && (uint64_t)nvert != 3ull * ntri)
        return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "an unindexed soup needs nvert == 3*ntri (%u vs %u)",
                    nvert, ntri);
    if (ntri > SLOTH_MAX_TRIANGLES) return fail(ctx, SLOTH_ERR_LIMIT, "too many triangles");
    if (idx)
        for (uint64_t i = 0; i < 3ull * ntri; ++i)
            if (idx[i] >= nvert)
                return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "index %u at %llu is out of range (nvert %u)",
                            idx[i], (unsigned long long)i, nvert);
    CU(ctx, cudaSetDevice(ctx->device));
    sloth_mesh *m = new sloth_mesh();
    m->ctx = ctx;
    m->device = ctx->device;
    m->nvert = nvert;
    m->ntri = ntri;
    auto cleanup = [&](sloth_status st) {
        sloth_mesh_destroy(m);
        return st;
    };
    if (dalloc(&m->x, nvert) || dalloc(&m->y, nvert) || dalloc(&m->z, nvert) ||
        dalloc(&m->rgb, 3 * (size_t)ntri) || (idx && dalloc(&m->idx, 3 * (size_t)ntri)))
        return cleanup(fail(ctx, SLOTH_ERR_OUT_OF_MEMORY, "mesh allocation failed"));
    cudaError_t e = cudaSuccess;
    if (nvert) {
        e = cudaMemcpy(m->x, x, nvert * sizeof(float), cudaMemcpyHostToDevice);
        if (!e) e = cudaMemcpy(m->y, y, nvert * sizeof(float), cudaMemcpyHostToDevice);
        if (!e) e = cudaMemcpy(m->z, z, nvert * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (!e && ntri) e = cudaMemcpy(m->rgb, rgb, 3 * (size_t)ntri, cudaMemcpyHostToDevice);
    if (!e && idx && ntri) e = cudaMemcpy(m->idx, idx, 3 * (size_t)ntri * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e) return cleanup(fail(ctx, SLOTH_ERR_CUDA, "mesh upload failed: %s", cudaGetErrorString(e)));
    // setup's spatial order (optional: without host memory for it the mesh keeps its own)
    std::vector<uint32_t> ord, oi;
    if (idx && ntri > 1) {
        try {
            spatial_order(x, y, z, idx, ntri, ord);
            oi.resize(3 * (size_t)ntri);
            for (uint32_t p = 0; p < ntri; ++p)
                for (int k = 0; k < 3; ++k) oi[3 * (size_t)p + k] = idx[3 * (size_t)ord[p] + k];
        } catch (const std::bad_alloc &) {
            ord.clear();
            oi.clear();
        }
    }
    if (!ord.empty() && (dalloc(&m->order, ntri) || dalloc(&m->oidx, 3 * (size_t)ntri))) {
        // no device memory for it: the mesh keeps its own order
        dfree(m->order);
        dfree(m->oidx);
        cudaGetLastError();
        ord.clear();
    }
    if (!ord.empty()) {
        e = cudaMemcpy(m->order, ord.data(), ntri * sizeof(uint32_t), cudaMemcpyHostToDevice);
        if (!e) e = cudaMemcpy(m->oidx, oi.data(), oi.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
        if (e) return cleanup(fail(ctx, SLOTH_ERR_CUDA, "mesh upload failed: %s", cudaGetErrorString(e)));
    }
    if (bbox_max) {
        memcpy(m->bbox_max, bbox_max, sizeof m->bbox_max);
    } else {
        // OBJ loader rule (src/geometry.rs:86-89,128-135): a box grown from the origin over
        // every triangle's vertices.
        float b[3] = {0.0f, 0.0f, 0.0f};
        const float *xyz[3] = {x, y, z};
        for (uint64_t t = 0; t < ntri; ++t)
            for (int k = 0; k < 3; ++k) {
                const uint64_t vi = idx ? idx[3 * t + k] : 3 * t + k;
                for (int c = 0; c < 3; ++c) b[c] = std::fmax(xyz[c][vi], b[c]);
            }
        memcpy(m->bbox_max, b, sizeof b);
    }
    ctx->meshes.push_back(m);
    *out = m;
    return SLOTH_OK;
}

void sloth_mesh_destroy(sloth_mesh *m)
{
    if (!m) return;
    if (m->ctx) {
        auto &v = m->ctx->meshes;
        v.erase(std::remove(v.begin(), v.end(), m), v.end());
    }
    cudaSetDevice(m->device);
    dfree(m->x);
    dfree(m->y);
    dfree(m->z);
    dfree(m->idx);
    dfree(m->rgb);
    dfree(m->order);
    dfree(m->oidx);
    delete m;
}

sloth_status sloth_mesh_update(sloth_mesh *m, const float *x, const float *y, const float *z,
                               const uint8_t *rgb)
{
    if (!m || !m->ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    sloth_ctx *ctx = m->ctx;
    if (m->nvert && (!x || !y || !z)) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "vertex arrays are NULL");
    if (m->ntri && !rgb) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "rgb is NULL");
    CU(ctx, cudaSetDevice(m->device));
    const size_t nb = (size_t)m->nvert * sizeof(float);
    if (m->nvert) {
        CU(ctx, cudaMemcpyAsync(m->x, x, nb, cudaMemcpyDefault, ctx->stream));
        CU(ctx, cudaMemcpyAsync(m->y, y, nb, cudaMemcpyDefault, ctx->stream));
        CU(ctx, cudaMemcpyAsync(m->z, z, nb, cudaMemcpyDefault, ctx->stream));
    }
    if (m->ntri) CU(ctx, cudaMemcpyAsync(m->rgb, rgb, 3 * (size_t)m->ntri, cudaMemcpyDefault, ctx->stream));
    return SLOTH_OK;
}

sloth_status sloth_mesh_info(const sloth_mesh *m, uint32_t *ntri, float bbox_max[3])
{
    if (!m) return SLOTH_ERR_INVALID_ARGUMENT;
    if (ntri) *ntri = m->ntri;
    if (bbox_max) memcpy(bbox_max, m->bbox_max, sizeof m->bbox_max);
    return SLOTH_OK;
}

// ---------------------------------------------------------------------------------------
// draw_mesh
// ---------------------------------------------------------------------------------------

// Grows the tile-entry buffer once the device has reported (without the host waiting for
// it) a draw whose entries exceeded it: such a draw was rasterized by the overflow
// fallback, and the later ones get a buffer that fits.  The growth itself waits for the
// context's stream (it frees the old buffer); it happens rarely, as the buffer doubles.
static sloth_status poll_entry_max(sloth_ctx *ctx)
{
    if (!ctx->max_pending) return SLOTH_OK;
    const cudaError_t q = cudaEventQuery(ctx->max_ev);
    if (q == cudaErrorNotReady) return SLOTH_OK;
    ctx->max_pending = false;
    CU(ctx, q);
    if (ctx->bb.entries && *ctx->h_max > ctx->bb.capacity) {
        size_t ecap = ctx->bb.capacity;
        sloth_status st = ensure_scratch(ctx, &ctx->bb.entries, &ecap, *ctx->h_max);
        if (st != SLOTH_OK) return st;
        ctx->bb.capacity = (uint32_t)(ecap > 0xffffffffu ? 0xffffffffu : ecap);
    }
    return SLOTH_OK;
}

sloth_status sloth_draw_mesh(sloth_ctx *ctx, const sloth_mesh *mesh, const float transform[16])
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    if (!mesh || !transform) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "mesh or transform is NULL");
    if (mesh->device != ctx->device) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "mesh is on another device");
    if (!ctx->have_frame) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "call sloth_ctx_clear before drawing");
    if (mesh->ntri == 0) return SLOTH_OK;
    if ((uint64_t)ctx->tri_base + mesh->ntri > SLOTH_MAX_TRIANGLES)
        return fail(ctx, SLOTH_ERR_LIMIT, "more than %u triangles since the last clear", SLOTH_MAX_TRIANGLES);
    CU(ctx, cudaSetDevice(ctx->device));
    sloth_status st;
    if ((st = poll_entry_max(ctx)) != SLOTH_OK) return st;
    if ((st = ensure_records(ctx, (size_t)ctx->tri_base + mesh->ntri)) != SLOTH_OK) return st;
    if (mesh->idx && (st = ensure_scratch(ctx, &ctx->tv, &ctx->tv_cap, mesh->nvert)) != SLOTH_OK) return st;
    if ((st = ensure_scratch(ctx, &ctx->bb.large_queue, &ctx->large_cap, mesh->ntri)) != SLOTH_OK) return st;
    if ((st = ensure_scratch(ctx, &ctx->bb.fill_list, &ctx->fill_cap, mesh->ntri)) != SLOTH_OK) return st;
    if (!ctx->bb.large_count) CU(ctx, dalloc(&ctx->bb.large_count, 3));
    ctx->bb.large_cap = mesh->ntri;

    Mat4 M;
    sloth_mat4_mul(ctx->U, transform, M.m);
    MeshDev md{mesh->x, mesh->y, mesh->z, mesh->idx, mesh->rgb, mesh->nvert, mesh->ntri, mesh->order, mesh->oidx};
    const FrameGeom &g = ctx->g;
    const uint32_t ntiles = (uint32_t)(g.ntx * g.nty);
    cudaStream_t s = ctx->stream;
    if ((st = join_newline(ctx)) != SLOTH_OK) return st;
    if ((st = apply_resets(ctx, true)) != SLOTH_OK) return st;
    // indexed meshes share vertices: transformed once by the vertex kernel; soups in setup
    const float4 *tv = mesh->idx ? ctx->tv : nullptr;
    if (tv) CU(ctx, timed(ctx, "vertex", [&] { return launch_vertex_transform(md, M, ctx->tv, s); }));
    CU(ctx, timed(ctx, "setup", [&] { return launch_setup(md, tv, M, ctx->tri_base, g, ctx->fb, ctx->bb, s, ctx->tpb); }));
    // the newline fold reads the records and feeds only the resolve: on its own stream,
    // beside the binning kernels
    CU(ctx, cudaEventRecord(ctx->setup_ev, s));
    CU(ctx, cudaStreamWaitEvent(ctx->nl_stream, ctx->setup_ev, 0));
    CU(ctx, timed(ctx, "newline", [&] { return launch_newline(mesh->ntri, mesh->order, ctx->tri_base, g, ctx->fb, ctx->nl_stream); },
                  ctx->nl_stream));
    CU(ctx, cudaEventRecord(ctx->nl_ev, ctx->nl_stream));
    ctx->nl_pending = true;
    CU(ctx, timed(ctx, "bin_count_large",[&] { return launch_bin_count_large(ctx->tri_base, g, ctx->fb, ctx->bb, s); }));
    CU(ctx, timed(ctx, "bin_scan", [&] { return launch_bin_scan(ntiles, ctx->bb, s); }));
    // The entry count is known only on the device.  With an entry buffer from earlier draws
    // the rest of the draw goes ahead with it and the host does not wait: the fill kernels
    // write no slot past the capacity, and when the count is above it the raster launch
    // folds the draw's binned triangles straight into the keys instead of rasterizing tiles
    // (the same keys).  The device's running maximum of the counts comes back on
    // a side stream, and a later draw grows the buffer from it (poll_entry_max).  The first
    // draw on a context, with no buffer yet, waits for its count and sizes the buffer.
    auto rest = [&](size_t entries_bound) -> sloth_status {
        // the small and the large fill take slots from the same cursors (atomics): they
        // run side by side, the large one on the aux stream
        CU(ctx, cudaEventRecord(ctx->fill_ev, s));
        CU(ctx, cudaStreamWaitEvent(ctx->aux, ctx->fill_ev, 0));
        CU(ctx, timed(ctx, "bin_fill_large", [&] { return launch_bin_fill_large(ctx->tri_base, g, ctx->fb, ctx->bb, ctx->aux); },
                      ctx->aux));
        CU(ctx, cudaEventRecord(ctx->aux_ev, ctx->aux));
        CU(ctx, timed(ctx, "bin_fill", [&] {
               return launch_bin_fill(ctx->tri_base, g, ctx->fb, ctx->bb, s);
           }));
        CU(ctx, cudaStreamWaitEvent(s, ctx->aux_ev, 0));
        size_t icap = ctx->bb.item_capacity;
        sloth_status st2;
        if ((st2 = ensure_scratch(ctx, &ctx->bb.items, &icap, raster_item_bound(ntiles, entries_bound))) != SLOTH_OK)
            return st2;
        ctx->bb.item_capacity = (uint32_t)icap;
        CU(ctx, timed(ctx, "bin_items", [&] { return launch_bin_items(ntiles, g, ctx->fb, ctx->bb, s); }));
        CU(ctx, timed(ctx, "raster", [&] {
               return launch_raster(g, ctx->fb, ctx->bb, ctx->depth_cull, mesh->ntri, ctx->tri_base, s);
           }));
        return SLOTH_OK;
    };
    if (ctx->bb.entries && ctx->bb.capacity > 0) {
        if ((st = rest(ctx->bb.capacity)) != SLOTH_OK) return st;
        if (!ctx->max_pending) {
            CU(ctx, cudaEventRecord(ctx->scan_ev, s));
            CU(ctx, cudaStreamWaitEvent(ctx->side, ctx->scan_ev, 0));
            CU(ctx, cudaMemcpyAsync(ctx->h_max, ctx->d_max, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->side));
            CU(ctx, cudaEventRecord(ctx->max_ev, ctx->side));
            ctx->max_pending = true;
        }
    } else {
        CU(ctx, cudaEventRecord(ctx->scan_ev, s));
        CU(ctx, cudaStreamWaitEvent(ctx->side, ctx->scan_ev, 0));
        CU(ctx, cudaMemcpyAsync(ctx->h_total, ctx->bb.tile_offset + ntiles, sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, ctx->side));
        CU(ctx, cudaEventRecord(ctx->total_ev, ctx->side));
        CU(ctx, cudaEventSynchronize(ctx->total_ev));
        const uint32_t total = *ctx->h_total;
        size_t ecap = ctx->bb.capacity;
        if ((st = ensure_scratch(ctx, &ctx->bb.entries, &ecap, total)) != SLOTH_OK) return st;
        ctx->bb.capacity = (uint32_t)(ecap > 0xffffffffu ? 0xffffffffu : ecap);
        if ((st = rest(total)) != SLOTH_OK) return st;
    }
    ctx->tri_base += mesh->ntri;
    ctx->dirty = true;
    return SLOTH_OK;
}

// ---------------------------------------------------------------------------------------
// timing hooks
// ---------------------------------------------------------------------------------------
sloth_status sloth_ctx_set_option(sloth_ctx *ctx, int option, int64_t value)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    switch (option) {
    case SLOTH_OPTION_TILE_SHAPE:
        if (value < 0 || value >= kNumTileShapes) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "no tile shape %lld", (long long)value);
        ctx->tile_shape = (int)value;
        return SLOTH_OK;
    case SLOTH_OPTION_WAIT_TEST:
        if (value != 0 && value != 1) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "wait test is 0 or 1");
        ctx->fb.wait_test = (uint32_t)value;
        return SLOTH_OK;
    case SLOTH_OPTION_DEPTH_CULL:
        if (value != 0 && value != 1) return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "depth cull is 0 or 1");
        ctx->depth_cull = (int)value;
        return SLOTH_OK;
    case SLOTH_OPTION_TRIANGLES_PER_BLOCK:
        if (!valid_triangles_per_block(value))
            return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "triangles per block %lld is not 128, 256, 1024 or 4096",
                        (long long)value);
        ctx->tpb = (int)value;
        return SLOTH_OK;
    case SLOTH_OPTION_DIRECT_SAMPLES:
        if (value < 0 || value > SLOTH_MAX_DIRECT_SAMPLES)
            return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "direct samples %lld outside 0..%d", (long long)value,
                        SLOTH_MAX_DIRECT_SAMPLES);
        ctx->direct_max = (int)value;
        return SLOTH_OK;
    default:
        return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "unknown option %d", option);
    }
}

// Candidate direct-sample limits of the single-frame autotuner.
static const int kCtxDirectCandidates[] = {0, 4, 16, 64};

sloth_status sloth_ctx_autotune(sloth_ctx *ctx, const sloth_mesh *const *meshes, const float *transforms,
                                uint32_t ndraws, int reps, int *best_shape, int *best_direct, int *best_tpb,
                                float *best_ms)
{
    if (!ctx || (ndraws && (!meshes || !transforms))) return SLOTH_ERR_INVALID_ARGUMENT;
    if (ctx->req_w == 0 || ctx->req_h == 0)
        return fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "no viewport: call sloth_ctx_set_viewport first");
    if (reps < 1) reps = 3;
    CU(ctx, cudaSetDevice(ctx->device));
    const int shape0 = ctx->tile_shape, direct0 = ctx->direct_max, tpb0 = ctx->tpb;
    const bool timing0 = ctx->timing;
    ctx->timing = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CU(ctx, cudaEventCreate(&e0));
    CU(ctx, cudaEventCreate(&e1));
    auto frame = [&]() -> sloth_status {
        sloth_status st = sloth_ctx_clear(ctx);
        for (uint32_t i = 0; i < ndraws && st == SLOTH_OK; ++i) st = sloth_draw_mesh(ctx, meshes[i], transforms + 16 * i);
        if (st == SLOTH_OK) st = resolve_pending(ctx);
        return st;
    };
    int bs = shape0, bd = direct0, bt = tpb0;
    float best = -1.0f;
    sloth_status st = SLOTH_OK;
    for (int shape = 0; shape < kNumTileShapes && st == SLOTH_OK; ++shape)
        for (int direct : kCtxDirectCandidates)
            for (int tpb : kTrianglesPerBlockChoices) {
                if (st != SLOTH_OK) break;
                ctx->tile_shape = shape;
                ctx->direct_max = direct;
                ctx->tpb = tpb;
                st = frame();                          // sizes buffers for this setting
                if (st == SLOTH_OK) st = sloth_ctx_synchronize(ctx);
                if (st == SLOTH_OK) st = frame();      // warm
                if (st != SLOTH_OK) break;
                cudaEventRecord(e0, ctx->stream);
                for (int r = 0; r < reps && st == SLOTH_OK; ++r) st = frame();
                cudaEventRecord(e1, ctx->stream);
                if (st == SLOTH_OK) st = sloth_ctx_synchronize(ctx);
                float ms = 0.0f;
                if (st == SLOTH_OK && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) {
                    ms /= (float)reps;
                    if (best < 0.0f || ms < best) {
                        best = ms;
                        bs = shape;
                        bd = direct;
                        bt = tpb;
                    }
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->timing = timing0;
    if (st != SLOTH_OK) {
        ctx->tile_shape = shape0;
        ctx->direct_max = direct0;
        ctx->tpb = tpb0;
        return st;
    }
    ctx->tile_shape = bs;
    ctx->direct_max = bd;
    ctx->tpb = bt;
    if (best_shape) *best_shape = bs;
    if (best_direct) *best_direct = bd;
    if (best_tpb) *best_tpb = bt;
    if (best_ms) *best_ms = best;
    return SLOTH_OK;
}

sloth_status sloth_ctx_set_timing(sloth_ctx *ctx, int enable)
{
    if (!ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    ctx->timing = enable != 0;
    return SLOTH_OK;
}

sloth_status sloth_ctx_kernel_time(sloth_ctx *ctx, const char *name, double *ms, uint64_t *launches)
{
    if (!ctx || !name) return SLOTH_ERR_INVALID_ARGUMENT;
    CU(ctx, cudaSetDevice(ctx->device));
    auto it = ctx->clocks.find(name);
    if (it == ctx->clocks.end()) {
        if (ms) *ms = 0.0;
        if (launches) *launches = 0;
        return SLOTH_OK;
    }
    KernelClock &kc = it->second;
    for (auto &ev : kc.pending) {
        CU(ctx, cudaEventSynchronize(ev.b));
        float t = 0.0f;
        CU(ctx, cudaEventElapsedTime(&t, ev.a, ev.b));
        kc.ms += t;
        kc.launches++;
        cudaEventDestroy(ev.a);
        cudaEventDestroy(ev.b);
    }
    kc.pending.clear();
    if (ms) *ms = kc.ms;
    if (launches) *launches = kc.launches;
    return SLOTH_OK;
}

uint64_t sloth_ctx_launch_count(const sloth_ctx *ctx) { return ctx ? ctx->launches : 0; }

}  // extern "C"
