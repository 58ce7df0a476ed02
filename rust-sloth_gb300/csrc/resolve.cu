// resolve.cu -- depth keys -> depth buffer, frame cells and winners (one frame).
// The per-cell rule is in resolve_common.cuh.
#include "resolve_common.cuh"

namespace sloth {

// Pairs of frame cells; each warp takes 32 consecutive pairs (resolve_pair).
__global__ void __launch_bounds__(256) resolve_kernel(FrameGeom g, FrameBuffers fb)
{
    const uint64_t nz = (uint64_t)g.w * g.h;
    const uint64_t ncells = g.image ? nz + g.h : nz;
    const uint64_t npairs = (ncells + 1) / 2;
    const int lane = threadIdx.x & 31;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < npairs; base += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = base + threadIdx.x;
        resolve_pair(g, fb, p, p < npairs, lane);
    }
}

cudaError_t launch_resolve(const FrameGeom &g, const FrameBuffers &fb, cudaStream_t s)
{
    const uint64_t ncells = (uint64_t)g.w * g.h + (g.image ? g.h : 0);
    if (ncells == 0) return cudaSuccess;
    uint64_t blocks = ((ncells + 1) / 2 + 255) / 256;
    if (blocks > 152u * 32u) blocks = 152u * 32u;
    resolve_kernel<<<(unsigned)blocks, 256, 0, s>>>(g, fb);
    return cudaGetLastError();
}

}  // namespace sloth
