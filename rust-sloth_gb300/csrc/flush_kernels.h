// flush_kernels.h -- GPU formatting of frame cells into Context::flush's bytes.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sloth {

// The three outputs of Context::flush(color, webify) (src/context.rs:50-92).
constexpr int kFlushPlain = 0;   // color false
constexpr int kFlushAnsi = 1;    // color true, webify false (crossterm 24-bit colour)
constexpr int kFlushHtml = 2;    // color true, webify true (HTML spans)

uint32_t flush_chunks(uint64_t ncells);       // entries of the chunk_bytes scratch
uint64_t flush_max_bytes(uint64_t ncells);    // an upper bound of the output size

// Formats ncells cells into out (device, at least flush_max_bytes(ncells) bytes) and
// writes the exact size to *size (device); chunk_bytes: flush_chunks(ncells) entries.
cudaError_t launch_flush(const uint32_t *cells, uint64_t ncells, int image, int format, uint64_t *chunk_bytes,
                         uint64_t *size, char *out, cudaStream_t s);

// Device scratch and output of the formatter, owned by a context or a batch.
struct FlushScratch {
    uint64_t *chunks = nullptr;
    size_t chunks_cap = 0;
    char *out = nullptr;          // the formatted bytes of the last flush
    size_t out_cap = 0;
    uint64_t *size_d = nullptr;   // device: output size
    uint64_t *size_h = nullptr;   // pinned host copy
};

// Format the cells into f.out and return the byte count (waits for the stream).
cudaError_t flush_run(FlushScratch &f, const uint32_t *cells, uint64_t ncells, int image, int format,
                      cudaStream_t s, uint64_t *bytes);
void flush_release(FlushScratch &f);

}  // namespace sloth
