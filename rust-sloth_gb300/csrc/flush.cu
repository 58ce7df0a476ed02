// flush.cu -- the bytes Context::flush prints, formatted on the GPU from the frame cells.
//
// src/context.rs:50-92.  For a frame of cells (char | r<<8 | g<<16 | b<<24):
//   - terminal contexts (image false) first queue crossterm's MoveTo(0,0): ESC "[1;1H";
//   - color false: every char, then println's "\n";
//   - color true, webify false: per cell crossterm 0.18's PrintStyledContent of the char
//     with foreground Rgb(r,g,b) on background Rgb(25,25,25):
//       ESC "[48;2;25;25;25m" ESC "[38;2;<r>;<g>;<b>m" <char> ESC "[0m"
//     (crossterm 0.18.0 is the version Cargo.lock pins; its source is not in the reference
//     tree, so this sequence restates its published StyledContent output: background,
//     foreground, content, ResetColor);
//   - color true, webify true: per cell "<span style=\"color:rgb(<r>,<g>,<b>)\"><char>".
// Numbers are decimal without padding.
//
// Three launches: per-chunk byte counts, one block scanning the chunk counts, and the
// formatter, which builds each chunk's text in shared memory and writes it out in one
// contiguous run.
#include <cstdint>

#include "flush_kernels.h"
#include "sloth_internal.cuh"

namespace sloth {

namespace {

constexpr int kFlushThreads = 256;
constexpr int kFlushCellsPerThread = 4;
constexpr uint32_t kFlushChunk = kFlushThreads * kFlushCellsPerThread;   // cells per block
constexpr uint32_t kMaxCellBytes = 40;                                      // ANSI: 31 + 9 digits

__device__ __forceinline__ uint32_t ndigits(uint32_t v) { return v >= 100 ? 3u : (v >= 10 ? 2u : 1u); }

__device__ __forceinline__ uint32_t cell_bytes(uint32_t cell, int format)
{
    if (format == kFlushPlain) return 1;
    const uint32_t d = ndigits((cell >> 8) & 255u) + ndigits((cell >> 16) & 255u) + ndigits(cell >> 24);
    return format == kFlushAnsi ? 31u + d : 29u + d;
}

__device__ __forceinline__ uint32_t put_str(char *o, const char *s)
{
    uint32_t n = 0;
    while (s[n]) {
        o[n] = s[n];
        ++n;
    }
    return n;
}

__device__ __forceinline__ uint32_t put_u8(char *o, uint32_t v)
{
    if (v >= 100) {
        o[0] = (char)('0' + v / 100);
        o[1] = (char)('0' + (v / 10) % 10);
        o[2] = (char)('0' + v % 10);
        return 3;
    }
    if (v >= 10) {
        o[0] = (char)('0' + v / 10);
        o[1] = (char)('0' + v % 10);
        return 2;
    }
    o[0] = (char)('0' + v);
    return 1;
}

__device__ __forceinline__ uint32_t put_cell(char *o, uint32_t cell, int format)
{
    const char ch = (char)(cell & 255u);
    if (format == kFlushPlain) {
        o[0] = ch;
        return 1;
    }
    const uint32_t r = (cell >> 8) & 255u, g = (cell >> 16) & 255u, b = cell >> 24;
    uint32_t n = 0;
    if (format == kFlushAnsi) {
        n += put_str(o + n, "\x1b[48;2;25;25;25m\x1b[38;2;");
        n += put_u8(o + n, r);
        o[n++] = ';';
        n += put_u8(o + n, g);
        o[n++] = ';';
        n += put_u8(o + n, b);
        o[n++] = 'm';
        o[n++] = ch;
        n += put_str(o + n, "\x1b[0m");
    } else {
        n += put_str(o + n, "<span style=\"color:rgb(");
        n += put_u8(o + n, r);
        o[n++] = ',';
        n += put_u8(o + n, g);
        o[n++] = ',';
        n += put_u8(o + n, b);
        o[n++] = ')';
        o[n++] = '"';
        o[n++] = '>';
        o[n++] = ch;
    }
    return n;
}

// Block-wide exclusive scan of one value per thread; returns the prefix, *total the sum.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *ws, uint32_t *total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += o;
    }
    if (lane == 31) ws[wid] = x;
    block_sync();
    if (wid == 0) {
        uint32_t s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, s, d);
            if (lane >= d) s += o;
        }
        ws[lane] = s;
    }
    block_sync();
    *total = ws[(blockDim.x >> 5) - 1];
    const uint32_t pre = x - v + (wid > 0 ? ws[wid - 1] : 0u);
    block_sync();   // ws may be reused by the caller
    return pre;
}

__global__ void __launch_bounds__(kFlushThreads)
flush_count_kernel(const uint32_t *__restrict__ cells, uint64_t ncells, int format, uint64_t *__restrict__ chunk_bytes)
{
    __shared__ uint32_t ws[32];
    const uint64_t c0 = (uint64_t)blockIdx.x * kFlushChunk + (uint64_t)threadIdx.x * kFlushCellsPerThread;
    uint32_t n = 0;
#pragma unroll
    for (int k = 0; k < kFlushCellsPerThread; ++k)
        if (c0 + k < ncells) n += cell_bytes(cells[c0 + k], format);
    uint32_t total;
    block_exclusive_scan(n, ws, &total);
    if (threadIdx.x == 0) chunk_bytes[blockIdx.x] = total;
}

// One block: exclusive scan of the chunk byte counts in place (64-bit), then the total
// output size (prefix + chunks + trailing newline) into *size.
__global__ void __launch_bounds__(1024)
flush_scan_kernel(uint64_t *__restrict__ chunk_bytes, uint32_t nchunks, uint32_t prefix, uint32_t suffix,
                  uint64_t *__restrict__ size)
{
    __shared__ unsigned long long ws[32];
    __shared__ unsigned long long carry;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = prefix;
    block_sync();
    for (uint32_t base = 0; base < nchunks; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const unsigned long long v = i < nchunks ? chunk_bytes[i] : 0ull;
        unsigned long long x = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long o = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += o;
        }
        if (lane == 31) ws[wid] = x;
        block_sync();
        if (wid == 0) {
            unsigned long long s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0ull;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned long long o = __shfl_up_sync(0xffffffffu, s, d);
                if (lane >= d) s += o;
            }
            ws[lane] = s;
        }
        block_sync();
        const unsigned long long pre = carry + x - v + (wid > 0 ? ws[wid - 1] : 0ull);
        if (i < nchunks) chunk_bytes[i] = pre;
        block_sync();
        if (threadIdx.x == blockDim.x - 1) carry = pre + v;
        block_sync();
    }
    if (threadIdx.x == 0) *size = carry + suffix;
}

// Each block formats its chunk into shared memory, then copies it out.
__global__ void __launch_bounds__(kFlushThreads)
flush_write_kernel(const uint32_t *__restrict__ cells, uint64_t ncells, int format,
                   const uint64_t *__restrict__ chunk_off, char *__restrict__ out)
{
    __shared__ uint32_t ws[32];
    __shared__ char text[kFlushChunk * kMaxCellBytes];
    const uint64_t c0 = (uint64_t)blockIdx.x * kFlushChunk + (uint64_t)threadIdx.x * kFlushCellsPerThread;
    uint32_t cv[kFlushCellsPerThread];
    uint32_t n = 0;
#pragma unroll
    for (int k = 0; k < kFlushCellsPerThread; ++k) {
        cv[k] = c0 + k < ncells ? cells[c0 + k] : 0u;
        if (c0 + k < ncells) n += cell_bytes(cv[k], format);
    }
    uint32_t total;
    uint32_t off = block_exclusive_scan(n, ws, &total);
#pragma unroll
    for (int k = 0; k < kFlushCellsPerThread; ++k)
        if (c0 + k < ncells) off += put_cell(text + off, cv[k], format);
    block_sync();
    char *dst = out + chunk_off[blockIdx.x];
    for (uint32_t i = threadIdx.x; i < total; i += blockDim.x) dst[i] = text[i];
}

__global__ void flush_ends_kernel(char *__restrict__ out, const uint64_t *__restrict__ size, int image, int suffix)
{
    if (threadIdx.x != 0) return;
    if (!image) {
        out[0] = '\x1b';
        out[1] = '[';
        out[2] = '1';
        out[3] = ';';
        out[4] = '1';
        out[5] = 'H';
    }
    if (suffix) out[*size - 1] = '\n';
}

}  // namespace

uint32_t flush_chunks(uint64_t ncells)
{
    return (uint32_t)((ncells + kFlushChunk - 1) / kFlushChunk);
}

uint64_t flush_max_bytes(uint64_t ncells)
{
    return 6 + ncells * kMaxCellBytes + 1;
}

cudaError_t launch_flush(const uint32_t *cells, uint64_t ncells, int image, int format, uint64_t *chunk_bytes,
                         uint64_t *size, char *out, cudaStream_t s)
{
    const uint32_t nch = flush_chunks(ncells);
    const uint32_t prefix = image ? 0u : 6u;
    const uint32_t suffix = format == kFlushPlain ? 1u : 0u;
    if (nch) flush_count_kernel<<<nch, kFlushThreads, 0, s>>>(cells, ncells, format, chunk_bytes);
    flush_scan_kernel<<<1, 1024, 0, s>>>(chunk_bytes, nch, prefix, suffix, size);
    if (nch) flush_write_kernel<<<nch, kFlushThreads, 0, s>>>(cells, ncells, format, chunk_bytes, out);
    flush_ends_kernel<<<1, 32, 0, s>>>(out, size, image, (int)suffix);
    return cudaGetLastError();
}

cudaError_t flush_run(FlushScratch &f, const uint32_t *cells, uint64_t ncells, int image, int format,
                      cudaStream_t s, uint64_t *bytes)
{
    cudaError_t e;
    const size_t nch = flush_chunks(ncells);
    const size_t need = flush_max_bytes(ncells);
    if (!f.size_d) {
        if ((e = cudaMalloc(&f.size_d, sizeof(uint64_t))) != cudaSuccess) return e;
        if ((e = cudaMallocHost(&f.size_h, sizeof(uint64_t))) != cudaSuccess) return e;
    }
    if (nch > f.chunks_cap || !f.chunks) {
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        if (f.chunks) cudaFree(f.chunks);
        f.chunks = nullptr;
        if ((e = cudaMalloc(&f.chunks, (nch ? nch : 1) * sizeof(uint64_t))) != cudaSuccess) return e;
        f.chunks_cap = nch;
    }
    if (need > f.out_cap || !f.out) {
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        if (f.out) cudaFree(f.out);
        f.out = nullptr;
        if ((e = cudaMalloc(&f.out, need)) != cudaSuccess) return e;
        f.out_cap = need;
    }
    if ((e = launch_flush(cells, ncells, image, format, f.chunks, f.size_d, f.out, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(f.size_h, f.size_d, sizeof(uint64_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    *bytes = *f.size_h;
    return cudaSuccess;
}

void flush_release(FlushScratch &f)
{
    if (f.chunks) cudaFree(f.chunks);
    if (f.out) cudaFree(f.out);
    if (f.size_d) cudaFree(f.size_d);
    if (f.size_h) cudaFreeHost(f.size_h);
    f = FlushScratch{};
}

}  // namespace sloth
