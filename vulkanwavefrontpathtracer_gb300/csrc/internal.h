// Host-only internals shared by the C ABI translation units.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/wfpt.h"
#include "scene.h"

namespace wfpt {

// Device status word bits (kErrTimeout / kErrBounds in common.cuh).
constexpr uint32_t kStatusTimeout = 1u;
constexpr uint32_t kStatusBounds = 2u;

wfpt_status from_cuda(cudaError_t e);
void set_error(const char* msg);

const SceneDevice* scene_device(const wfpt_scene* s);
bool scene_has(const wfpt_scene* s, int kind);
void scene_bounds(const wfpt_scene* s, float mn[3], float mx[3]);

// Renderer allocation fault injection (renderer.cpp).
void set_fail_alloc_after(int n);
int get_fail_alloc_after();
// Shadow batch slots of the renderer's memory planner (0 = planned).
void set_shadow_slots(int n);
int get_shadow_slots();

}  // namespace wfpt
