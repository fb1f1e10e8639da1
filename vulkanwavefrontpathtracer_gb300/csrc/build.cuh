// Device build of the acceleration structures (build.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace wfpt {

// Device buffers of a device-built scene (all owned by the caller after the
// build; free with cudaFree).
struct DeviceBuild {
    void* bvh2_nodes = nullptr;  // Bvh2Node[bvh2_count]
    void* bvh2_tris = nullptr;   // TriRec[num_triangles]
    void* bvh8_nodes = nullptr;  // Bvh8Node[bvh8_count]
    void* bvh8_tris = nullptr;   // TriRec[num_triangles]
    uint32_t bvh2_count = 0, bvh8_count = 0;
    float bounds_min[3] = {0, 0, 0}, bounds_max[3] = {0, 0, 0};
    uint32_t ploc_iterations = 0;
};

// Builds the BVH2 (PLOC over 63-bit Morton-sorted triangle centroids,
// single-triangle leaves) and, when want8, the BVH8 by the SAH collapse
// (same policy knobs as the host collapse) from device-resident geometry:
// positions_dev float[3*num_vertices], indices_dev uint32[3*num_triangles],
// geom_first_dev uint32[num_geoms] (ascending, first 0).  Needs at least two
// triangles.  Synchronises `s` between PLOC iterations and BVH8 levels.
// Returns cudaErrorInvalidValue when a triangle index is out of range.
cudaError_t build_scene_device(const float* positions_dev, uint32_t num_vertices, const uint32_t* indices_dev,
                               uint32_t num_triangles, const uint32_t* geom_first_dev, uint32_t num_geoms,
                               bool want8, cudaStream_t s, DeviceBuild* out);

cudaError_t status_build(uint32_t* out);
// PLOC search radius, 1..64 clusters on either side (default 8).
void set_ploc_radius(int r);
int get_ploc_radius();

}  // namespace wfpt
