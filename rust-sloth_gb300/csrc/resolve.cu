// resolve.cu -- depth keys -> depth buffer, frame cells and winners (one frame).
// The per-cell rule is in resolve_common.cuh.
#include "resolve_common.cuh"

namespace sloth {

// Runs of kRun frame cells; each warp takes 32 consecutive runs (resolve_run).  An
// even-width frame goes by pairs of cells instead, kEvenPairs per thread (resolve_even).
constexpr int kRun = 2;
constexpr int kEvenPairs = 4;

__global__ void __launch_bounds__(256, 4) resolve_kernel(FrameGeom g, FrameBuffers fb, int vec)
{
    const uint64_t nz = (uint64_t)g.w * g.h;
    const uint64_t ncells = g.image ? nz + g.h : nz;
    if (!(g.w & 1)) {
        const uint64_t npairs = (ncells + 1) / 2, span = (uint64_t)blockDim.x * kEvenPairs;
        for (uint64_t base = blockIdx.x * span; base < npairs; base += (uint64_t)gridDim.x * span)
            resolve_even<kEvenPairs>(g, fb, base + threadIdx.x, blockDim.x, npairs, vec != 0);
        return;
    }
    const uint64_t nruns = (ncells + kRun - 1) / kRun;
    const int lane = threadIdx.x & 31;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < nruns; base += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = base + threadIdx.x;
        resolve_run<kRun>(g, fb, p, p < nruns, lane, vec != 0);
    }
}

cudaError_t launch_resolve(const FrameGeom &g, const FrameBuffers &fb, cudaStream_t s)
{
    const uint64_t ncells = (uint64_t)g.w * g.h + (g.image ? g.h : 0);
    if (ncells == 0) return cudaSuccess;
    const uint64_t per_block = 256ull * kRun * ((g.w & 1) ? 1 : kEvenPairs);   // cells
    uint64_t blocks = (ncells + per_block - 1) / per_block;
    const uint64_t cap = 32ull * (uint64_t)device_sm_count();   // four resident CTAs per SM (64 registers), eight waves
    if (blocks > cap) blocks = cap;
    const int vec = ((reinterpret_cast<uintptr_t>(fb.cells_out) | reinterpret_cast<uintptr_t>(fb.z_out) |
                      reinterpret_cast<uintptr_t>(fb.winner_out)) & (4u * kRun - 1u)) == 0;
    resolve_kernel<<<(unsigned)blocks, 256, 0, s>>>(g, fb, vec);
    return cudaGetLastError();
}

}  // namespace sloth
