// noalloc.cu -- sloth_render_noalloc: one frame of one triangle soup with no device
// allocation.
//
// Some callers cannot let a library call cudaMalloc:
//  - hosts that give the renderer a fixed memory budget at start-up and forbid
//    allocation afterwards (plug-ins, embedded viewers);
//  - frame loops that cannot afford the device-wide synchronisation cudaMalloc/cudaFree
//    imply;
//  - programs whose device memory is fully reserved by a framework's caching pool.
// For them this entry point takes device inputs and outputs from the caller and keeps
// every intermediate buffer in one file-scope __device__ array of a fixed size
// (kScratchBytes).  That array exists on every GPU that loads the library, until the
// process exits.  It has no counterpart in the reference.
//
// Scratch layout (byte offsets into g_noalloc_scratch):
//   records   kMaxTri x 96 B          per-triangle setup records
//   rows      kMaxTri x 4 B           per-triangle packed sample rows (setup -> newline)
//   keys      kMaxCells x 8 B         depth keys (tiles padded to 64x32 cells)
//   bins      tile counts/offsets/cursors, the large-triangle queue and its counter
//   tile_gen  kMaxTiles x 4 B         tile generations (cleared every call)
//   nltree    2*kMaxNl x 4 B          newline segment tree (cleared every call)
//   frags     8 B                     fragment counter (cleared every call)
#include "sloth_gpu.h"
#include "sloth_internal.cuh"
#include "sloth_kernels.h"

namespace sloth {
namespace {

constexpr uint32_t kMaxTri = SLOTH_NOALLOC_MAX_TRIANGLES;
constexpr uint32_t kMaxCells = SLOTH_NOALLOC_MAX_DEPTH_CELLS;
constexpr uint32_t kMaxNl = SLOTH_NOALLOC_MAX_HEIGHT;            // power of two
constexpr uint32_t kMaxTiles = kMaxCells / (kTileW * kTileH);

constexpr size_t align256(size_t n) { return (n + 255) & ~size_t(255); }
constexpr size_t kOffRecords = 0;
constexpr size_t kOffRows = align256(kOffRecords + (size_t)kMaxTri * sizeof(TriRecord));
constexpr size_t kOffKeys = align256(kOffRows + (size_t)kMaxTri * 4);
constexpr size_t kOffCount = align256(kOffKeys + (size_t)kMaxCells * sizeof(uint64_t));
constexpr size_t kOffOffset = align256(kOffCount + (size_t)kMaxTiles * 4);
constexpr size_t kOffCursor = align256(kOffOffset + ((size_t)kMaxTiles + 1) * 4);
constexpr size_t kOffQueue = align256(kOffCursor + (size_t)kMaxTiles * 4);
constexpr size_t kOffQCount = align256(kOffQueue + (size_t)kMaxTri * 4);
constexpr size_t kOffGen = align256(kOffQCount + 8);
constexpr size_t kOffNl = align256(kOffGen + (size_t)kMaxTiles * 4);
constexpr size_t kOffFrags = align256(kOffNl + 2 * (size_t)kMaxNl * 4);
constexpr size_t kScratchBytes = align256(kOffFrags + 8);
static_assert(kScratchBytes == SLOTH_NOALLOC_SCRATCH_BYTES, "header states the scratch size");

}  // namespace

// The scratch every call uses.  In host code this name is only a stand-in for the
// device symbol; its device address comes from cudaGetSymbolAddress (scratch_on()), with
// the device the caller made current.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Raster variant without binning: one CTA per tile tests every triangle of the draw
// against the tile (the soup is bounded by kMaxTri) and folds covered samples' depth
// keys into a shared-memory tile with the same 64-bit atomicMin as raster_kernel.
__global__ void __launch_bounds__(256)
noalloc_raster_kernel(uint32_t ntri, FrameGeom g, FrameBuffers fb)
{
    constexpr int TW = kTileW, TH = kTileH;
    __shared__ unsigned long long skeys[TH * TW];
    __shared__ uint32_t s_next, s_frags[8];
    const int tile = blockIdx.x;
    const int tr = tile / g.ntx, tc = tile - tr * g.ntx;
    const int R0 = tr * TH, C0 = tc * TW;
    for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) skeys[i] = kEmptyKey;
    if (threadIdx.x == 0) s_next = 0;
    block_sync();
    const int lane = threadIdx.x & 31;
    const Viewport vp{g.w, g.h, g.image, g.tw, g.th, g.ntx, g.nty, g.pitch};
    uint32_t frags = 0;
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(&s_next, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntri) break;
        const TriRecord r = fb.records[t];
        const Rect U = unwrapped_part(vp, r.x0, r.xe, r.y0, r.y1);
        const Rect W = wrapped_part(vp, r.x0, r.xe, r.y0, r.y1);
        const Rect cu = U.empty() ? Rect{0, 0, 0, 0} : clip_unwrapped(vp, U, tr, tc);
        const Rect cw = W.empty() ? Rect{0, 0, 0, 0} : clip_wrapped(vp, W, tr, tc);
        const bool exact = (r.flags & kFlagFiniteXY) != 0;
        for (int part = 0; part < 2; ++part) {
            const Rect c = part == 0 ? cu : cw;
            if (c.empty() || (exact && !rect_may_cover(r, c))) continue;
            const int bw = c.xb - c.xa, area = bw * (c.yb - c.ya);
            for (int k = lane; k < area; k += 32) {
                const int x = c.xa + k % bw, y = c.ya + k / bw;
                const EdgeVals e = eval_edges(r, (float)x, (float)y);
                if (e.w0 >= 0.0f && e.w1 >= 0.0f && e.w2 >= 0.0f) {
                    ++frags;
                    const float z = interp_z(r.v1z, r.dz2, r.dz3, r.a, e.w1, e.w2);
                    if (z < kFltMax) {
                        const uint32_t nw = part == 0 ? 1u : 0u;
                        const unsigned long long key = make_key(z, t, nw);
                        const int row = nw ? (y - R0) : (y + 1 - R0);
                        const int col = nw ? (2 * x - C0) : (2 * x - g.w - C0);
                        unsigned long long *p = &skeys[row * TW + key_col(col, TW)];
                        if (key < *(volatile unsigned long long *)p) atomicMin(p, key);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) frags += __shfl_xor_sync(0xffffffffu, frags, d);
    if (lane == 0) s_frags[threadIdx.x >> 5] = frags;
    block_sync();
    unsigned long long *gk = reinterpret_cast<unsigned long long *>(fb.keys) + (size_t)R0 * g.pitch + C0;
    // shared and global keys share the layout (key_col): slot i of tile row rr is slot i globally
    for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
        const int rr = i / TW, cc = i - rr * TW;
        gk[(size_t)rr * g.pitch + cc] = skeys[i];
    }
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int k = 0; k < 8; ++k) tot += s_frags[k];
        atomicAdd(fb.fragments, (unsigned long long)tot);
        fb.tile_gen[tile] = fb.gen;
    }
}

namespace {

// Device address of g_noalloc_scratch for the current device, looked up on every call with
// the caller's device current.  cudaGetSymbolAddress allocates nothing; an address kept
// from an earlier call could belong to a context that cudaDeviceReset (or a driver-API
// caller switching contexts) has since replaced, and kernels given it would fault.
cudaError_t scratch_on(unsigned char **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    *out = static_cast<unsigned char *>(p);
    return cudaSuccess;
}

}  // namespace
}  // namespace sloth

using namespace sloth;

extern "C" sloth_status sloth_render_noalloc(const float *x, const float *y, const float *z,
                                             uint32_t ntri, const uint8_t *rgb, const float m[16],
                                             uint32_t width, uint32_t height, int image,
                                             uint32_t *cells, float *zbuf, int32_t *winner, void *stream)
{
    if (!m || !cells || !zbuf || !winner || (ntri && (!x || !y || !z || !rgb)))
        return SLOTH_ERR_INVALID_ARGUMENT;
    if (width < 1 || height < 1 || width > SLOTH_MAX_DIM || height > SLOTH_NOALLOC_MAX_HEIGHT)
        return SLOTH_ERR_LIMIT;
    if (ntri > kMaxTri) return SLOTH_ERR_LIMIT;
    FrameGeom g{};
    g.w = (int32_t)width;
    g.h = (int32_t)height;
    g.image = image ? 1 : 0;
    g.tw = kTileW;
    g.th = kTileH;
    g.ntx = (g.w + g.tw - 1) / g.tw;
    g.nty = (g.h + g.th - 1) / g.th;
    g.pitch = g.ntx * g.tw;
    g.nl_size = 1;
    while (g.nl_size < g.h) g.nl_size <<= 1;
    const uint64_t padded = (uint64_t)g.pitch * g.nty * g.th;
    if (padded > kMaxCells) return SLOTH_ERR_LIMIT;
    const uint32_t ntiles = (uint32_t)(g.ntx * g.nty);

    unsigned char *base = nullptr;
    if (scratch_on(&base) != cudaSuccess) return SLOTH_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    FrameBuffers fb{};
    fb.records = reinterpret_cast<TriRecord *>(base + kOffRecords);
    fb.rows = reinterpret_cast<uint32_t *>(base + kOffRows);
    fb.keys = reinterpret_cast<uint64_t *>(base + kOffKeys);
    fb.tile_gen = reinterpret_cast<uint32_t *>(base + kOffGen);
    fb.nltree = reinterpret_cast<int32_t *>(base + kOffNl);
    fb.fragments = reinterpret_cast<unsigned long long *>(base + kOffFrags);
    fb.z_out = zbuf;
    fb.cells_out = cells;
    fb.winner_out = winner;
    fb.gen = 1;
    BinBuffers bb{};
    bb.tile_count = reinterpret_cast<uint32_t *>(base + kOffCount);
    bb.tile_offset = reinterpret_cast<uint32_t *>(base + kOffOffset);
    bb.tile_cursor = reinterpret_cast<uint32_t *>(base + kOffCursor);
    bb.large_queue = reinterpret_cast<uint32_t *>(base + kOffQueue);
    bb.large_count = reinterpret_cast<uint32_t *>(base + kOffQCount);
    bb.large_cap = kMaxTri;
    bb.entries = nullptr;
    bb.capacity = 0;

    // The array keeps the previous call's contents: reset what must start empty.
    cudaError_t e;
    if ((e = cudaMemsetAsync(fb.tile_gen, 0, ntiles * sizeof(uint32_t), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(fb.nltree, 0xff, 2 * (size_t)g.nl_size * sizeof(int32_t), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(fb.fragments, 0, sizeof(unsigned long long), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(bb.tile_count, 0, ntiles * sizeof(uint32_t), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(bb.large_count, 0, 2 * sizeof(uint32_t), s)) != cudaSuccess)
        return SLOTH_ERR_CUDA;
    Mat4 M;
    for (int i = 0; i < 16; ++i) M.m[i] = m[i];
    MeshDev md{x, y, z, nullptr, rgb, 3 * ntri, ntri};
    if (launch_setup(md, nullptr, M, 0, g, fb, bb, s) != cudaSuccess) return SLOTH_ERR_CUDA;
    if (launch_newline(ntri, nullptr, 0, g, fb, s) != cudaSuccess) return SLOTH_ERR_CUDA;
    if (ntri) {
        noalloc_raster_kernel<<<ntiles, 256, 0, s>>>(ntri, g, fb);
        if (cudaGetLastError() != cudaSuccess) return SLOTH_ERR_CUDA;
    }
    if (launch_resolve(g, fb, s) != cudaSuccess) return SLOTH_ERR_CUDA;
    return SLOTH_OK;
}
