// Traversal launch wrapper.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/wfpt.h"
#include "scene.h"

namespace wfpt {

cudaError_t launch_trace(const SceneDevice& sc, int kind, const wfpt_ray* rays, wfpt_hit* results,
                         const uint32_t* ray_index, uint32_t n, const uint32_t* n_dev, int closest,
                         cudaStream_t s);

}  // namespace wfpt
