// diff_kernels.h -- launchers of the differentiable shading of a rendered batch.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "batch_kernels.h"

namespace sloth {

constexpr uint32_t kDiffChunk = 2048;   // depth cells (or samples) per block

// blocks[i] = (frame, first depth cell), chunks of kDiffChunk over w*h per frame; the
// same table walks the w*h samples (x in [0,w), y in [0,h)) of the backward pass.
cudaError_t launch_batch_shade(const BatchDev &b, const int2 *blocks, uint32_t nblocks, const float *vrgb,
                               const float *light, float *rgb, uint2 *vis, cudaStream_t s);
cudaError_t launch_batch_shade_backward(const BatchDev &b, const int2 *blocks, uint32_t nblocks, const float *vrgb,
                                        const float *light, const float *grad_rgb, const uint2 *vis, float *gpos,
                                        float *gcol, float *glight, cudaStream_t s);

}  // namespace sloth
