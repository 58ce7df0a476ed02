// batch_api.cu -- sloth_batch_*: many frames, views and meshes per launch sequence.
//
// The reference renders one frame at a time (src/main.rs:60-111: update, clear, draw
// every mesh of the queue, flush); its multi-frame export (`image -j N`) and multi-model
// queues repeat that loop.  A batch holds many such frames at once -- each with its own
// viewport, image mode, utransform and ordered draws -- and renders all of them with one
// pass of each kernel and one persistent raster pass over a device-side (frame, tile)
// queue.  After the first render (which sizes the tile-entry buffer on the host) the
// whole sequence is captured in a CUDA graph and replayed.  If a later render's entries
// outgrow the buffer, the raster reports it and the next read re-plans and re-renders.
#include <cstring>
#include <string>
#include <vector>

#include "batch_kernels.h"
#include "diff_kernels.h"
#include "flush_kernels.h"
#include "sloth_gpu.h"
#include "sloth_internal.cuh"

using namespace sloth;

// Clear generation of every batch frame: each render clears the tile generations to 0 (no
// tile current) or, when small triangles are folded straight into the keys, fills them
// with the byte 0x01 (every tile current), so the value has 0x01 in every byte.
constexpr uint32_t kBatchGen = 0x01010101u;

struct sloth_batch {
    sloth_ctx *ctx = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<sloth_frame_desc> frames;
    std::vector<const sloth_mesh *> meshes;   // per draw
    std::vector<float> transforms;            // 16 per draw
    int shape = 0;
    int direct_max = 0;                       // FrameGeom::direct_max of every frame
    bool persistent = true;                   // raster over the device queue (else one CTA per item)
    int tpb = kDefaultTrianglesPerBlock;      // triangles per setup block

    // layout (per shape)
    std::vector<BatchFrame> hframes;
    std::vector<uint64_t> cell_off, z_off;    // per frame
    uint32_t total_tiles = 0;
    uint64_t total_cells = 0, total_z = 0, total_keys = 0, total_nl = 0, total_rec = 0, total_vert = 0;
    // runs of consecutive frames' keys with the same width parity: (first key, keys, even width)
    struct KeyRun {
        uint64_t off, n;
        bool even;
    };
    std::vector<KeyRun> key_runs;
    int max_nl = 1;

    // device memory
    BatchFrame *d_frames = nullptr;
    BatchDraw *d_draws = nullptr;
    Mat4 *d_mats = nullptr;
    Mat4 *h_mats = nullptr;                   // pinned
    float4 *tv = nullptr;                     // transformed vertices: written for shading only (want_tv)
    TriRecord *records = nullptr;
    uint32_t *rows = nullptr;                 // packed sample rows per record (setup -> newline)
    uint64_t *keys = nullptr;
    uint32_t *tile_gen = nullptr;
    int32_t *nltree = nullptr;
    float *z = nullptr;
    uint32_t *cells = nullptr;
    int32_t *winner = nullptr;
    unsigned long long *fragments = nullptr;
    uint32_t *frame_tile_off = nullptr;
    BinBuffers bb{};
    size_t entries_cap = 0;
    uint32_t *large_frame = nullptr;
    uint32_t *overflow = nullptr;
    uint32_t *queue = nullptr;                // the persistent raster's item counter
    uint4 *fill_list = nullptr;               // the fill's work list (one entry per record at most)
    uint32_t *fill_count = nullptr;
    uint32_t *h_total = nullptr;              // pinned
    uint32_t *h_overflow = nullptr;           // pinned
    uint32_t *error = nullptr;                // device error word of the raster (sticky)
    uint32_t *h_error = nullptr;              // pinned
    int2 *blk[4] = {nullptr, nullptr, nullptr, nullptr};   // vertex, triangle, newline, resolve
    uint32_t nblk[4] = {0, 0, 0, 0};

    cudaGraphExec_t graph = nullptr;
    bool rendered = false;
    // side branches of a render: the newline fold (beside the binning) and the
    // large-triangle fill (beside the small one), forked from and joined into `stream`
    cudaStream_t nl_s = nullptr, aux_s = nullptr;
    cudaEvent_t ev_setup = nullptr, ev_nl = nullptr, ev_fill = nullptr, ev_aux = nullptr;

    // differentiable shading
    int2 *diff_blk = nullptr;                 // (frame, first depth cell) per kDiffChunk
    uint32_t ndiff_blk = 0;
    uint2 *vis = nullptr;                     // stored visibility, one per depth cell
    bool vis_valid = false;                   // vis holds the last render's visibility
    bool want_tv = false;                     // shading has been used: renders fill tv

    FlushScratch flush;
};

// Shared with sloth_api.cu.
extern "C++" {
sloth_status sloth_ctx_fail(sloth_ctx *ctx, sloth_status st, const char *msg);
void sloth_ctx_register_batch(sloth_ctx *ctx, sloth_batch *b);
void sloth_ctx_unregister_batch(sloth_ctx *ctx, sloth_batch *b);
int sloth_ctx_device(const sloth_ctx *ctx);
cudaStream_t sloth_ctx_stream(const sloth_ctx *ctx);
int sloth_ctx_depth_cull(const sloth_ctx *ctx);
int sloth_ctx_direct_samples(const sloth_ctx *ctx);
struct MeshView {
    const float *x, *y, *z;
    const uint32_t *idx;
    const uint8_t *rgb;
    uint32_t nvert, ntri;
    int device;
    const uint32_t *order, *oidx;   // setup's order of an indexed mesh (MeshDev), or null
};
MeshView sloth_mesh_view(const sloth_mesh *m);
}

namespace {

#define BCU(b, call)                                                                           \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return sloth_ctx_fail((b)->ctx, e_ == cudaErrorMemoryAllocation ? SLOTH_ERR_OUT_OF_MEMORY \
                                                                            : SLOTH_ERR_CUDA,  \
                                  (std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
    } while (0)

template <class T>
cudaError_t balloc(T **p, size_t n)
{
    *p = nullptr;
    return cudaMalloc(reinterpret_cast<void **>(p), (n ? n : 1) * sizeof(T));
}
template <class T>
void bfree(T *&p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

void free_layout(sloth_batch *b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    bfree(b->d_frames);
    bfree(b->d_draws);
    bfree(b->d_mats);
    bfree(b->tv);
    bfree(b->records);
    bfree(b->rows);
    bfree(b->keys);
    bfree(b->tile_gen);
    bfree(b->nltree);
    bfree(b->z);
    bfree(b->cells);
    bfree(b->winner);
    bfree(b->fragments);
    bfree(b->frame_tile_off);
    bfree(b->bb.tile_count);
    bfree(b->bb.tile_offset);
    bfree(b->bb.tile_cursor);
    bfree(b->bb.entries);
    bfree(b->bb.large_queue);
    bfree(b->bb.large_count);
    bfree(b->large_frame);
    bfree(b->bb.slice_offset);
    bfree(b->bb.items);
    b->bb.item_capacity = 0;
    bfree(b->overflow);
    bfree(b->queue);
    bfree(b->fill_list);
    bfree(b->fill_count);
    for (auto &p : b->blk) bfree(p);
    b->entries_cap = 0;
    b->rendered = false;
}

void set_mats(sloth_batch *b)
{
    for (size_t f = 0; f < b->frames.size(); ++f) {
        const sloth_frame_desc &fd = b->frames[f];
        for (uint32_t k = 0; k < fd.ndraws; ++k) {
            const uint32_t d = fd.first_draw + k;
            sloth_mat4_mul(fd.utransform, &b->transforms[16 * (size_t)d], b->h_mats[d].m);
        }
    }
}

// Lay out every frame for tile shape `shape` and allocate the batch's buffers.
sloth_status build(sloth_batch *b, int shape)
{
    free_layout(b);
    b->vis_valid = false;
    b->shape = shape;
    const int tw = kTileShapes[shape][0], th = kTileShapes[shape][1];
    const uint32_t nf = (uint32_t)b->frames.size(), nd = (uint32_t)b->meshes.size();
    b->hframes.assign(nf, BatchFrame{});
    b->key_runs.clear();
    b->cell_off.assign(nf + 1, 0);
    b->z_off.assign(nf + 1, 0);
    std::vector<uint64_t> key_off(nf), nl_off(nf), rec_off(nf);
    std::vector<uint32_t> tile_off(nf + 1, 0);
    std::vector<BatchDraw> hd(nd);
    uint64_t keys = 0, nl = 0, rec = 0, vert = 0, cells = 0, zs = 0;
    uint32_t tiles = 0;
    b->max_nl = 1;
    std::vector<int2> bv, bt, bn, br;
    for (uint32_t f = 0; f < nf; ++f) {
        const sloth_frame_desc &fd = b->frames[f];
        FrameGeom g{};
        g.w = (int32_t)fd.width;
        g.h = (int32_t)fd.height;
        g.image = fd.image ? 1 : 0;
        g.tw = tw;
        g.th = th;
        g.ntx = (g.w + tw - 1) / tw;
        g.nty = (g.h + th - 1) / th;
        g.pitch = g.ntx * tw;
        g.nl_size = 1;
        while (g.nl_size < g.h) g.nl_size <<= 1;
        g.direct_max = b->direct_max;
        b->max_nl = g.nl_size > b->max_nl ? g.nl_size : b->max_nl;
        BatchFrame &bf = b->hframes[f];
        bf.g = g;
        bf.tile_off = tiles;
        bf.rec_off = (uint32_t)rec;
        bf.first_draw = fd.first_draw;
        bf.ndraws = fd.ndraws;
        bf.z_off = zs;
        tile_off[f] = tiles;
        key_off[f] = keys;
        {
            const uint64_t nk = (uint64_t)g.pitch * g.nty * th;
            const bool even = !(g.w & 1);
            if (!b->key_runs.empty() && b->key_runs.back().even == even) b->key_runs.back().n += nk;
            else b->key_runs.push_back({keys, nk, even});
        }
        nl_off[f] = nl;
        rec_off[f] = rec;
        b->cell_off[f] = cells;
        b->z_off[f] = zs;
        tiles += (uint32_t)(g.ntx * g.nty);
        keys += (uint64_t)g.pitch * g.nty * th;
        nl += 2 * (uint64_t)g.nl_size;
        const uint64_t nz = (uint64_t)g.w * g.h;
        cells += g.image ? nz + g.h : nz;
        zs += nz;
        uint32_t local = 0;
        for (uint32_t k = 0; k < fd.ndraws; ++k) {
            const uint32_t d = fd.first_draw + k;
            const MeshView mv = sloth_mesh_view(b->meshes[d]);
            BatchDraw &bd = hd[d];
            bd.mesh = MeshDev{mv.x, mv.y, mv.z, mv.idx, mv.rgb, mv.nvert, mv.ntri, mv.order, mv.oidx};
            bd.frame = f;
            bd.rec_off = (uint32_t)(rec + local);
            bd.local_base = local;
            bd.vert_off = (uint32_t)vert;
            for (uint32_t q = 0; q < (mv.nvert + 3) / 4; q += 256) bv.push_back(make_int2((int)d, (int)q));
            for (uint32_t t = 0; t < mv.ntri; t += (uint32_t)b->tpb) bt.push_back(make_int2((int)d, (int)t));
            if (g.image)
                for (uint32_t t = 0; t < mv.ntri; t += kBatchNewlineChunk) bn.push_back(make_int2((int)d, (int)t));
            local += mv.ntri;
            vert += mv.nvert;
        }
        rec += local;
        const uint64_t nc = g.image ? nz + g.h : nz;
        for (uint64_t c = 0; c < nc; c += kBatchResolveChunk) br.push_back(make_int2((int)f, (int)c));
    }
    if (rec > 0x7fffffffull) return sloth_ctx_fail(b->ctx, SLOTH_ERR_LIMIT, "batch has more than 2^31 triangles");
    tile_off[nf] = tiles;
    b->cell_off[nf] = cells;
    b->z_off[nf] = zs;
    b->total_tiles = tiles;
    b->total_cells = cells;
    b->total_z = zs;
    b->total_keys = keys;
    b->total_nl = nl;
    b->total_rec = rec;
    b->total_vert = vert;

    BCU(b, balloc(&b->tv, vert));
    BCU(b, balloc(&b->records, rec));
    BCU(b, balloc(&b->rows, rec));
    BCU(b, balloc(&b->keys, keys));
    BCU(b, balloc(&b->tile_gen, tiles));
    BCU(b, balloc(&b->nltree, nl));
    BCU(b, balloc(&b->z, zs));
    BCU(b, balloc(&b->cells, cells));
    BCU(b, balloc(&b->winner, zs));
    BCU(b, balloc(&b->fragments, 1));
    BCU(b, balloc(&b->frame_tile_off, nf + 1));
    BCU(b, balloc(&b->bb.tile_count, tiles));
    BCU(b, balloc(&b->bb.tile_offset, tiles + 1));
    BCU(b, balloc(&b->bb.tile_cursor, tiles));
    BCU(b, balloc(&b->bb.large_queue, rec));
    BCU(b, balloc(&b->bb.large_count, 2));
    b->bb.large_cap = (uint32_t)rec;
    BCU(b, balloc(&b->large_frame, rec));
    BCU(b, balloc(&b->bb.slice_offset, tiles + kSliceExtra));
    BCU(b, balloc(&b->overflow, 1));
    BCU(b, balloc(&b->queue, 1));
    BCU(b, balloc(&b->fill_list, rec));
    BCU(b, balloc(&b->fill_count, 1));
    BCU(b, balloc(&b->d_mats, nd));
    for (uint32_t f = 0; f < nf; ++f) {
        BatchFrame &bf = b->hframes[f];
        bf.fb.keys = b->keys + key_off[f];
        bf.fb.tile_gen = b->tile_gen + tile_off[f];
        bf.fb.nltree = b->nltree + nl_off[f];
        bf.fb.records = b->records + rec_off[f];
        bf.fb.rows = b->rows + rec_off[f];
        bf.fb.z_out = b->z + b->z_off[f];
        bf.fb.cells_out = b->cells + b->cell_off[f];
        bf.fb.winner_out = b->winner + b->z_off[f];
        bf.vec = ((b->cell_off[f] | b->z_off[f]) & 1u) == 0;   // the buffers are 256-byte aligned
        bf.fb.fragments = b->fragments;
        bf.fb.error = b->error;
        bf.fb.gen = kBatchGen;
    }
    BCU(b, balloc(&b->d_frames, nf));
    BCU(b, balloc(&b->d_draws, nd));
    BCU(b, cudaMemcpy(b->d_frames, b->hframes.data(), nf * sizeof(BatchFrame), cudaMemcpyHostToDevice));
    BCU(b, cudaMemcpy(b->d_draws, hd.data(), nd * sizeof(BatchDraw), cudaMemcpyHostToDevice));
    BCU(b, cudaMemcpy(b->frame_tile_off, tile_off.data(), (nf + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice));
    std::vector<int2> *tabs[4] = {&bv, &bt, &bn, &br};
    for (int i = 0; i < 4; ++i) {
        b->nblk[i] = (uint32_t)tabs[i]->size();
        BCU(b, balloc(&b->blk[i], tabs[i]->size()));
        if (!tabs[i]->empty())
            BCU(b, cudaMemcpy(b->blk[i], tabs[i]->data(), tabs[i]->size() * sizeof(int2), cudaMemcpyHostToDevice));
    }
    return SLOTH_OK;
}

BatchDev dev_view(sloth_batch *b)
{
    BatchDev d{};
    d.frames = b->d_frames;
    d.draws = b->d_draws;
    d.mats = b->d_mats;
    d.tv = b->tv;
    d.nframes = (uint32_t)b->frames.size();
    d.ndraws = (uint32_t)b->meshes.size();
    d.total_tiles = b->total_tiles;
    d.frame_tile_off = b->frame_tile_off;
    d.bb = b->bb;
    d.bb.capacity = (uint32_t)(b->entries_cap > 0xffffffffu ? 0xffffffffu : b->entries_cap);
    d.large_frame = b->large_frame;
    d.overflow = b->overflow;
    d.queue = b->queue;
    d.fill_list = b->fill_list;
    d.fill_count = b->fill_count;
    d.depth_cull = sloth_ctx_depth_cull(b->ctx);
    d.tpb = b->tpb;
    d.direct_max = b->direct_max;
    return d;
}

// Stage 1: reset, matrices, vertices (once shading wants them), setup, newline, large
// counts, scan.
cudaError_t enqueue_front(sloth_batch *b, const BatchDev &d, cudaStream_t s)
{
    cudaError_t e;
    if ((e = cudaMemsetAsync(b->bb.tile_count, 0, (size_t)b->total_tiles * 4, s))) return e;
    if ((e = cudaMemsetAsync(b->bb.tile_cursor, 0, (size_t)b->total_tiles * 4, s))) return e;
    if (b->direct_max > 0) {
        // small triangles fold into the global keys during setup: every tile's keys start
        // empty and current (kBatchGen is 0x01 in every byte)
        for (const auto &kr : b->key_runs)
            if ((e = launch_clear_keys(b->keys + kr.off, kr.n, kTileShapes[b->shape][0], kr.even, s))) return e;
        if ((e = cudaMemsetAsync(b->tile_gen, 0x01, (size_t)b->total_tiles * 4, s))) return e;
    } else {
        if ((e = cudaMemsetAsync(b->tile_gen, 0, (size_t)b->total_tiles * 4, s))) return e;
    }
    if ((e = cudaMemsetAsync(b->nltree, 0xff, (size_t)b->total_nl * 4, s))) return e;
    if ((e = cudaMemsetAsync(b->bb.large_count, 0, 8, s))) return e;
    if ((e = cudaMemsetAsync(b->fill_count, 0, 4, s))) return e;
    if ((e = cudaMemsetAsync(b->fragments, 0, 8, s))) return e;
    if ((e = cudaMemsetAsync(b->overflow, 0, 4, s))) return e;
    if ((e = cudaMemcpyAsync(b->d_mats, b->h_mats, b->meshes.size() * sizeof(Mat4), cudaMemcpyHostToDevice, s)))
        return e;
    if (b->want_tv && (e = launch_batch_vertex(d, b->blk[0], b->nblk[0], s))) return e;
    if ((e = launch_batch_setup(d, b->blk[1], b->nblk[1], s))) return e;
    if ((e = cudaEventRecord(b->ev_setup, s))) return e;
    if ((e = cudaStreamWaitEvent(b->nl_s, b->ev_setup, 0))) return e;
    if ((e = launch_batch_newline(d, b->blk[2], b->nblk[2], b->max_nl, b->nl_s))) return e;
    if ((e = cudaEventRecord(b->ev_nl, b->nl_s))) return e;
    if ((e = launch_batch_bin_large(d, false, s))) return e;
    return launch_bin_scan(b->total_tiles, d.bb, s);
}

// Stage 2: fill, persistent raster, resolve.
cudaError_t enqueue_back(sloth_batch *b, const BatchDev &d, cudaStream_t s)
{
    cudaError_t e;
    if ((e = cudaEventRecord(b->ev_fill, s))) return e;
    if ((e = cudaStreamWaitEvent(b->aux_s, b->ev_fill, 0))) return e;
    if ((e = launch_batch_bin_large(d, true, b->aux_s))) return e;
    if ((e = cudaEventRecord(b->ev_aux, b->aux_s))) return e;
    if ((e = launch_batch_fill(d, s))) return e;
    if ((e = cudaStreamWaitEvent(s, b->ev_aux, 0))) return e;
    if ((e = launch_batch_items(d, s))) return e;
    const int tw = kTileShapes[b->shape][0], th = kTileShapes[b->shape][1];
    if ((e = launch_batch_raster(d, tw, th, b->persistent, s))) return e;
    if ((e = cudaStreamWaitEvent(s, b->ev_nl, 0))) return e;   // the newline tree is complete
    return launch_batch_resolve(d, b->blk[3], b->nblk[3], s);
}

// Render without the graph: stage 1, size the entries from the scan total, stage 2.
sloth_status render_planned(sloth_batch *b)
{
    cudaStream_t s = b->stream;
    BatchDev d = dev_view(b);
    BCU(b, enqueue_front(b, d, s));
    BCU(b, cudaMemcpyAsync(b->h_total, b->bb.tile_offset + b->total_tiles, 4, cudaMemcpyDeviceToHost, s));
    BCU(b, cudaStreamSynchronize(s));
    const size_t need = (size_t)*b->h_total;
    if (need > b->entries_cap || !b->bb.entries) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        bfree(b->bb.entries);
        bfree(b->bb.items);
        const size_t cap = need + need / 4 + 1024;   // headroom for other transforms
        BCU(b, balloc(&b->bb.entries, cap));
        b->entries_cap = cap;
        b->bb.item_capacity = raster_item_bound(b->total_tiles, cap);
        BCU(b, balloc(&b->bb.items, b->bb.item_capacity));
        d = dev_view(b);
    }
    BCU(b, enqueue_back(b, d, s));
    b->rendered = true;
    return SLOTH_OK;
}

sloth_status capture(sloth_batch *b)
{
    cudaStream_t s = b->stream;
    const BatchDev d = dev_view(b);
    cudaGraph_t g = nullptr;
    BCU(b, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_front(b, d, s);
    if (e == cudaSuccess) e = enqueue_back(b, d, s);
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return sloth_ctx_fail(b->ctx, SLOTH_ERR_CUDA, "batch graph capture failed");
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    BCU(b, e);
    return SLOTH_OK;
}

// After a render: if the entries outgrew their buffer, re-plan and re-render.
sloth_status settle(sloth_batch *b)
{
    BCU(b, cudaMemcpyAsync(b->h_overflow, b->overflow, 4, cudaMemcpyDeviceToHost, b->stream));
    BCU(b, cudaMemcpyAsync(b->h_error, b->error, 4, cudaMemcpyDeviceToHost, b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    if (*b->h_error)
        return sloth_ctx_fail(b->ctx, SLOTH_ERR_DEVICE_FAULT, "a raster block gave up waiting for its tile copy");
    if (*b->h_overflow) {
        sloth_status st = render_planned(b);
        if (st != SLOTH_OK) return st;
        BCU(b, cudaStreamSynchronize(b->stream));
    }
    return SLOTH_OK;
}

// Checks shared by the forward and backward shading calls; builds the block table.
sloth_status diff_prepare(sloth_batch *b, const float *vertex_rgb, const float *light)
{
    if (!vertex_rgb || !light) return sloth_ctx_fail(b->ctx, SLOTH_ERR_INVALID_ARGUMENT, "vertex_rgb/light are NULL");
    if (!b->rendered) return sloth_ctx_fail(b->ctx, SLOTH_ERR_INVALID_ARGUMENT, "render the batch first");
    for (const sloth_mesh *m : b->meshes)
        if (m != b->meshes[0])
            return sloth_ctx_fail(b->ctx, SLOTH_ERR_INVALID_ARGUMENT, "shading needs one mesh for every draw");
    BCU(b, cudaSetDevice(b->device));
    if (!b->diff_blk) {
        std::vector<int2> t;
        for (uint32_t f = 0; f < (uint32_t)b->frames.size(); ++f) {
            const uint64_t nz = b->z_off[f + 1] - b->z_off[f];
            for (uint64_t c = 0; c < nz; c += kDiffChunk) t.push_back(make_int2((int)f, (int)c));
        }
        BCU(b, balloc(&b->diff_blk, t.size()));
        if (!t.empty())
            BCU(b, cudaMemcpy(b->diff_blk, t.data(), t.size() * sizeof(int2), cudaMemcpyHostToDevice));
        b->ndiff_blk = (uint32_t)t.size();
    }
    // the keys of the last render must be complete (re-render if its entries overflowed)
    sloth_status st = settle(b);
    if (st != SLOTH_OK) return st;
    if (!b->want_tv) {
        // the first shading of this batch: transform the vertices the last render drew, and
        // let every later render do it too (the graph is captured again)
        BCU(b, launch_batch_vertex(dev_view(b), b->blk[0], b->nblk[0], b->stream));
        b->want_tv = true;
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
    }
    return SLOTH_OK;
}


}  // namespace

// Release a batch's device and pinned memory and cut it from its context (its context is
// being destroyed, or the batch is).  The handle stays valid for sloth_batch_destroy.
void sloth_batch_detach(sloth_batch *b)
{
    if (!b->ctx) return;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    if (b->nl_s) cudaStreamSynchronize(b->nl_s);
    if (b->aux_s) cudaStreamSynchronize(b->aux_s);
    free_layout(b);
    bfree(b->diff_blk);
    bfree(b->vis);
    flush_release(b->flush);
    if (b->h_mats) cudaFreeHost(b->h_mats);
    if (b->h_total) cudaFreeHost(b->h_total);
    if (b->h_overflow) cudaFreeHost(b->h_overflow);
    if (b->h_error) cudaFreeHost(b->h_error);
    bfree(b->error);
    for (cudaEvent_t *ev : {&b->ev_setup, &b->ev_nl, &b->ev_fill, &b->ev_aux})
        if (*ev) {
            cudaEventDestroy(*ev);
            *ev = nullptr;
        }
    for (cudaStream_t *st : {&b->nl_s, &b->aux_s})
        if (*st) {
            cudaStreamDestroy(*st);
            *st = nullptr;
        }
    b->h_mats = nullptr;
    b->h_total = b->h_overflow = b->h_error = nullptr;
    b->ctx = nullptr;
    b->stream = nullptr;
    b->rendered = false;
}

extern "C" {

sloth_status sloth_batch_create(sloth_ctx *ctx, const sloth_frame_desc *frames, uint32_t nframes,
                                const sloth_draw_desc *draws, uint32_t ndraws, sloth_batch **out)
{
    if (!ctx || !out || (nframes && !frames) || (ndraws && !draws)) return SLOTH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    for (uint32_t f = 0; f < nframes; ++f) {
        const sloth_frame_desc &fd = frames[f];
        if (fd.width < 1 || fd.height < 1 || fd.width > SLOTH_MAX_DIM || fd.height > SLOTH_MAX_DIM)
            return sloth_ctx_fail(ctx, SLOTH_ERR_LIMIT, "frame viewport outside 1..65535");
        if ((uint64_t)fd.first_draw + fd.ndraws > ndraws)
            return sloth_ctx_fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "frame draws outside the draw array");
        if (f > 0 && fd.first_draw != frames[f - 1].first_draw + frames[f - 1].ndraws)
            return sloth_ctx_fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "frames must list consecutive draw ranges");
    }
    if (nframes && frames[0].first_draw != 0)
        return sloth_ctx_fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "the first frame must start at draw 0");
    const int dev = sloth_ctx_device(ctx);
    for (uint32_t d = 0; d < ndraws; ++d) {
        if (!draws[d].mesh) return sloth_ctx_fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "draw without a mesh");
        if (sloth_mesh_view(draws[d].mesh).device != dev)
            return sloth_ctx_fail(ctx, SLOTH_ERR_INVALID_ARGUMENT, "mesh on another device");
    }
    if (cudaSetDevice(dev) != cudaSuccess) return SLOTH_ERR_CUDA;
    sloth_batch *b = new sloth_batch();
    b->ctx = ctx;
    b->device = dev;
    b->stream = sloth_ctx_stream(ctx);
    b->frames.assign(frames, frames + nframes);
    for (uint32_t d = 0; d < ndraws; ++d) {
        b->meshes.push_back(draws[d].mesh);
        b->transforms.insert(b->transforms.end(), draws[d].transform, draws[d].transform + 16);
    }
    if (cudaMallocHost(&b->h_mats, (ndraws ? ndraws : 1) * sizeof(Mat4)) != cudaSuccess ||
        cudaMallocHost(&b->h_total, 4) != cudaSuccess || cudaMallocHost(&b->h_overflow, 4) != cudaSuccess ||
        cudaMallocHost(&b->h_error, 4) != cudaSuccess || cudaMalloc(&b->error, 4) != cudaSuccess ||
        cudaMemset(b->error, 0, 4) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->nl_s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->aux_s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_setup, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_nl, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fill, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_aux, cudaEventDisableTiming) != cudaSuccess ||
        prepare_batch_kernels() != cudaSuccess) {
        sloth_batch_detach(b);
        delete b;
        return sloth_ctx_fail(ctx, SLOTH_ERR_OUT_OF_MEMORY, "batch host buffers");
    }
    sloth_ctx_register_batch(ctx, b);
    b->direct_max = sloth_ctx_direct_samples(ctx);
    set_mats(b);
    const sloth_status st = build(b, 0);
    if (st != SLOTH_OK) {
        sloth_batch_destroy(b);
        return st;
    }
    *out = b;
    return SLOTH_OK;
}

void sloth_batch_destroy(sloth_batch *b)
{
    if (!b) return;
    if (b->ctx) {
        sloth_ctx_unregister_batch(b->ctx, b);
        sloth_batch_detach(b);
    }
    delete b;
}

sloth_status sloth_batch_set_transforms(sloth_batch *b, const float *transforms)
{
    if (!b || !b->ctx || !transforms) return SLOTH_ERR_INVALID_ARGUMENT;
    BCU(b, cudaSetDevice(b->device));
    BCU(b, cudaStreamSynchronize(b->stream));   // the previous render has read the matrices
    memcpy(b->transforms.data(), transforms, b->transforms.size() * sizeof(float));
    set_mats(b);
    return SLOTH_OK;
}

sloth_status sloth_batch_render(sloth_batch *b)
{
    if (!b || !b->ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    BCU(b, cudaSetDevice(b->device));
    b->vis_valid = false;
    if (!b->rendered || !b->bb.entries) return render_planned(b);
    if (!b->graph && b->stream != nullptr) {
        const sloth_status st = capture(b);
        if (st != SLOTH_OK) return st;
    }
    if (b->graph) {
        BCU(b, cudaGraphLaunch(b->graph, b->stream));
        return SLOTH_OK;
    }
    return render_planned(b);
}

sloth_status sloth_batch_read(sloth_batch *b, uint32_t frame, uint32_t *cells, float *z, int32_t *winner)
{
    if (!b || !b->ctx || frame >= b->frames.size()) return SLOTH_ERR_INVALID_ARGUMENT;
    if (!b->rendered) return sloth_ctx_fail(b->ctx, SLOTH_ERR_INVALID_ARGUMENT, "render the batch first");
    BCU(b, cudaSetDevice(b->device));
    sloth_status st = settle(b);
    if (st != SLOTH_OK) return st;
    const uint64_t nc = b->cell_off[frame + 1] - b->cell_off[frame];
    const uint64_t nz = b->z_off[frame + 1] - b->z_off[frame];
    if (cells)
        BCU(b, cudaMemcpyAsync(cells, b->cells + b->cell_off[frame], nc * 4, cudaMemcpyDeviceToHost, b->stream));
    if (z) BCU(b, cudaMemcpyAsync(z, b->z + b->z_off[frame], nz * 4, cudaMemcpyDeviceToHost, b->stream));
    if (winner)
        BCU(b, cudaMemcpyAsync(winner, b->winner + b->z_off[frame], nz * 4, cudaMemcpyDeviceToHost, b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    return SLOTH_OK;
}

sloth_status sloth_batch_flush(sloth_batch *b, uint32_t frame, int format, char *out, uint64_t capacity,
                               uint64_t *bytes)
{
    if (!b || !b->ctx || frame >= b->frames.size() || !bytes) return SLOTH_ERR_INVALID_ARGUMENT;
    if (format < SLOTH_FLUSH_PLAIN || format > SLOTH_FLUSH_HTML)
        return sloth_ctx_fail(b->ctx, SLOTH_ERR_INVALID_ARGUMENT, "unknown flush format");
    if (!b->rendered) return sloth_ctx_fail(b->ctx, SLOTH_ERR_INVALID_ARGUMENT, "render the batch first");
    BCU(b, cudaSetDevice(b->device));
    sloth_status st = settle(b);
    if (st != SLOTH_OK) return st;
    const uint64_t nc = b->cell_off[frame + 1] - b->cell_off[frame];
    BCU(b, flush_run(b->flush, b->cells + b->cell_off[frame], nc, b->frames[frame].image ? 1 : 0, format, b->stream,
                     bytes));
    if (!out) return SLOTH_OK;
    if (capacity < *bytes) return sloth_ctx_fail(b->ctx, SLOTH_ERR_LIMIT, "flush output buffer too small");
    BCU(b, cudaMemcpyAsync(out, b->flush.out, *bytes, cudaMemcpyDeviceToHost, b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    return SLOTH_OK;
}

sloth_status sloth_batch_frame_buffers(sloth_batch *b, uint32_t frame, const uint32_t **cells, const float **z)
{
    if (!b || !b->ctx || frame >= b->frames.size()) return SLOTH_ERR_INVALID_ARGUMENT;
    if (cells) *cells = b->cells + b->cell_off[frame];
    if (z) *z = b->z + b->z_off[frame];
    return SLOTH_OK;
}

sloth_status sloth_batch_fragments(sloth_batch *b, uint64_t *fragments)
{
    if (!b || !b->ctx || !fragments) return SLOTH_ERR_INVALID_ARGUMENT;
    BCU(b, cudaSetDevice(b->device));
    sloth_status st = settle(b);
    if (st != SLOTH_OK) return st;
    unsigned long long v = 0;
    BCU(b, cudaMemcpy(&v, b->fragments, 8, cudaMemcpyDeviceToHost));
    *fragments = v;
    return SLOTH_OK;
}

sloth_status sloth_batch_set_tile_shape(sloth_batch *b, int shape)
{
    if (!b || !b->ctx || shape < 0 || shape >= kNumTileShapes) return SLOTH_ERR_INVALID_ARGUMENT;
    BCU(b, cudaSetDevice(b->device));
    BCU(b, cudaStreamSynchronize(b->stream));
    return shape == b->shape ? SLOTH_OK : build(b, shape);
}

sloth_status sloth_batch_set_triangles_per_block(sloth_batch *b, int tpb)
{
    if (!b || !b->ctx || !valid_triangles_per_block(tpb)) return SLOTH_ERR_INVALID_ARGUMENT;
    BCU(b, cudaSetDevice(b->device));
    BCU(b, cudaStreamSynchronize(b->stream));
    if (tpb == b->tpb) return SLOTH_OK;
    b->tpb = tpb;
    // the triangle block table steps by tpb: rebuild it
    std::vector<int2> bt;
    for (const sloth_frame_desc &fd : b->frames)
        for (uint32_t k = 0; k < fd.ndraws; ++k) {
            const uint32_t d = fd.first_draw + k;
            const uint32_t ntri = sloth_mesh_view(b->meshes[d]).ntri;
            for (uint32_t t = 0; t < ntri; t += (uint32_t)tpb) bt.push_back(make_int2((int)d, (int)t));
        }
    bfree(b->blk[1]);
    b->nblk[1] = (uint32_t)bt.size();
    BCU(b, balloc(&b->blk[1], bt.size()));
    if (!bt.empty()) BCU(b, cudaMemcpy(b->blk[1], bt.data(), bt.size() * sizeof(int2), cudaMemcpyHostToDevice));
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return SLOTH_OK;
}

sloth_status sloth_batch_set_persistent(sloth_batch *b, int persistent)
{
    if (!b || !b->ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    BCU(b, cudaSetDevice(b->device));
    BCU(b, cudaStreamSynchronize(b->stream));
    if ((persistent != 0) == b->persistent) return SLOTH_OK;
    b->persistent = persistent != 0;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);   // the raster launch is part of the graph
        b->graph = nullptr;
    }
    return SLOTH_OK;
}

sloth_status sloth_batch_set_direct_samples(sloth_batch *b, int samples)
{
    if (!b || !b->ctx || samples < 0 || samples > SLOTH_MAX_DIRECT_SAMPLES) return SLOTH_ERR_INVALID_ARGUMENT;
    BCU(b, cudaSetDevice(b->device));
    BCU(b, cudaStreamSynchronize(b->stream));
    if (samples == b->direct_max) return SLOTH_OK;
    b->direct_max = samples;
    for (BatchFrame &f : b->hframes) f.g.direct_max = samples;
    if (b->d_frames)
        BCU(b, cudaMemcpy(b->d_frames, b->hframes.data(), b->hframes.size() * sizeof(BatchFrame),
                          cudaMemcpyHostToDevice));
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);   // the key clear of a render depends on the setting
        b->graph = nullptr;
    }
    return SLOTH_OK;
}

// Candidate sample limits of the direct path the autotuner tries (0: every triangle binned).
static const int kDirectCandidates[] = {0, 4, 16, 64};

namespace {

// The batch's tuning state: (tile shape, direct limit, triangles per block, persistent).
struct BatchTune {
    int shape, direct, tpb, persistent;
};

sloth_status apply_tune(sloth_batch *b, const BatchTune &t)
{
    sloth_status st = sloth_batch_set_tile_shape(b, t.shape);
    if (st == SLOTH_OK) st = sloth_batch_set_direct_samples(b, t.direct);
    if (st == SLOTH_OK) st = sloth_batch_set_triangles_per_block(b, t.tpb);
    if (st == SLOTH_OK) st = sloth_batch_set_persistent(b, t.persistent);
    return st;
}

// Mean render time (ms) of `reps` graph replays with the given settings.
sloth_status time_tune(sloth_batch *b, const BatchTune &t, int reps, cudaEvent_t e0, cudaEvent_t e1, float *ms)
{
    sloth_status st = apply_tune(b, t);
    if (st == SLOTH_OK) st = sloth_batch_render(b);     // plan + size the entries
    if (st == SLOTH_OK) st = settle(b);
    if (st == SLOTH_OK) st = sloth_batch_render(b);     // capture + warm
    if (st == SLOTH_OK) st = settle(b);
    if (st != SLOTH_OK) return st;
    BCU(b, cudaEventRecord(e0, b->stream));
    for (int i = 0; i < reps && st == SLOTH_OK; ++i) st = sloth_batch_render(b);
    BCU(b, cudaEventRecord(e1, b->stream));
    BCU(b, cudaEventSynchronize(e1));
    if (st != SLOTH_OK) return st;
    BCU(b, cudaEventElapsedTime(ms, e0, e1));
    *ms /= (float)reps;
    return SLOTH_OK;
}

}  // namespace

sloth_status sloth_batch_autotune(sloth_batch *b, int reps, int *best_shape, int *best_direct, int *best_tpb,
                                  int *best_persistent, float *best_ms)
{
    if (!b || !b->ctx) return SLOTH_ERR_INVALID_ARGUMENT;
    if (reps < 1) reps = 3;
    BCU(b, cudaSetDevice(b->device));
    cudaEvent_t e0, e1;
    BCU(b, cudaEventCreate(&e0));
    BCU(b, cudaEventCreate(&e1));
    // coordinate descent from the current settings: each dimension in turn, twice over
    BatchTune best{b->shape, b->direct_max, b->tpb, b->persistent ? 1 : 0};
    float best_t = -1.0f;
    sloth_status st = time_tune(b, best, reps, e0, e1, &best_t);
    for (int round = 0; round < 2 && st == SLOTH_OK; ++round) {
        for (int dim = 0; dim < 4 && st == SLOTH_OK; ++dim) {
            const int n = dim == 0 ? kNumTileShapes : dim == 1 ? 4 : dim == 2 ? 4 : 2;
            BatchTune keep = best;
            for (int k = 0; k < n && st == SLOTH_OK; ++k) {
                BatchTune t = keep;
                if (dim == 0) t.shape = k;
                if (dim == 1) t.direct = kDirectCandidates[k];
                if (dim == 2) t.tpb = kTrianglesPerBlockChoices[k];
                if (dim == 3) t.persistent = k;
                if (t.shape == keep.shape && t.direct == keep.direct && t.tpb == keep.tpb &&
                    t.persistent == keep.persistent)
                    continue;
                float ms = 0.0f;
                st = time_tune(b, t, reps, e0, e1, &ms);
                if (st == SLOTH_OK && ms < best_t) {
                    best = t;
                    best_t = ms;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st == SLOTH_OK) st = apply_tune(b, best);
    if (st != SLOTH_OK) return st;
    if (best_shape) *best_shape = best.shape;
    if (best_direct) *best_direct = best.direct;
    if (best_tpb) *best_tpb = best.tpb;
    if (best_persistent) *best_persistent = best.persistent;
    if (best_ms) *best_ms = best_t;
    return SLOTH_OK;
}

// ---- differentiable shading -------------------------------------------------------

sloth_status sloth_batch_depth_cells(sloth_batch *b, uint32_t frame, uint64_t *first, uint64_t *count)
{
    if (!b || !b->ctx || frame >= b->frames.size()) return SLOTH_ERR_INVALID_ARGUMENT;
    if (first) *first = b->z_off[frame];
    if (count) *count = b->z_off[frame + 1] - b->z_off[frame];
    return SLOTH_OK;
}

sloth_status sloth_batch_shade(sloth_batch *b, const float *vertex_rgb, const float *light, float *rgb,
                               int store_visibility)
{
    if (!b || !b->ctx || !rgb) return SLOTH_ERR_INVALID_ARGUMENT;
    sloth_status st = diff_prepare(b, vertex_rgb, light);
    if (st != SLOTH_OK) return st;
    if (store_visibility && !b->vis) BCU(b, balloc(&b->vis, b->total_z));
    BCU(b, launch_batch_shade(dev_view(b), b->diff_blk, b->ndiff_blk, vertex_rgb, light, rgb,
                              store_visibility ? b->vis : nullptr, b->stream));
    b->vis_valid = store_visibility != 0;
    return SLOTH_OK;
}

sloth_status sloth_batch_shade_backward(sloth_batch *b, const float *vertex_rgb, const float *light,
                                        const float *grad_rgb, float *grad_pos, float *grad_vertex_rgb,
                                        float *grad_light)
{
    if (!b || !b->ctx || !grad_rgb) return SLOTH_ERR_INVALID_ARGUMENT;
    sloth_status st = diff_prepare(b, vertex_rgb, light);
    if (st != SLOTH_OK) return st;
    BCU(b, launch_batch_shade_backward(dev_view(b), b->diff_blk, b->ndiff_blk, vertex_rgb, light, grad_rgb,
                                       b->vis_valid ? b->vis : nullptr, grad_pos, grad_vertex_rgb, grad_light,
                                       b->stream));
    return SLOTH_OK;
}

sloth_status sloth_tile_shape(int shape, uint32_t *cells, uint32_t *rows)
{
    if (shape < 0 || shape >= kNumTileShapes) return SLOTH_ERR_INVALID_ARGUMENT;
    if (cells) *cells = (uint32_t)kTileShapes[shape][0];
    if (rows) *rows = (uint32_t)kTileShapes[shape][1];
    return SLOTH_OK;
}

}  // extern "C"
