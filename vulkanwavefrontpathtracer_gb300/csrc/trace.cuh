// Traversal launch wrapper.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/wfpt.h"
#include "scene.h"

namespace wfpt {

// Persistent BVH8 traversal refills a warp when at least this many lanes
// are idle (1..32; 32 = only when the whole warp is idle).
void set_trace_refill(uint32_t refill);
// Postpone a node's triangle tests while fewer than this many lanes of the
// warp have triangles to test (0 = never).
void set_trace_postpone(uint32_t lanes);
// Cooperative triangle tests: batch size and node steps per loop iteration,
// set separately for closest-hit and any-hit rays.
void set_trace_batch(uint32_t pairs, bool closest);
uint32_t get_trace_batch(bool closest);
void set_trace_steps(uint32_t steps, bool closest);
uint32_t get_trace_steps(bool closest);
uint32_t get_trace_refill();
uint32_t get_trace_postpone();
// Warp-cooperative triangle tests in the BVH8 traversal (on by default).
void set_trace_coop(bool on);
bool get_trace_coop();
// Counting variants of the traversal kernels (node visits, triangle tests,
// rays, persistent-warp iterations) for diagnostics.
void set_trace_count(bool on);
bool get_trace_count();
cudaError_t trace_counters(uint64_t out[4], bool reset);
cudaError_t trace_prepare();

// work (nullable): the persistent BVH8 kernel's two self-resetting work
// counters (zeroed once by the owner); launches that use the same counters
// must be ordered one after another.  Null takes the next of the scene's
// counter slots.
cudaError_t launch_trace(const SceneDevice& sc, int kind, const wfpt_ray* rays, wfpt_hit* results,
                         const uint32_t* ray_index, uint32_t n, const uint32_t* n_dev, int closest,
                         cudaStream_t s, uint32_t* work = nullptr);

}  // namespace wfpt
