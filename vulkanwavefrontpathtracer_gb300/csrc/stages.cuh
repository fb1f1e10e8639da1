// Launch wrappers of the stage kernels (host-callable, stream-ordered).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/wfpt.h"

namespace wfpt {

// Per-frame values read on the device by a captured frame graph (updated by
// one host-to-device copy before each launch).
struct FrameParams {
    float s2w[16];      // inverse(P * V), column-major
    float eye[3];
    float zfar;
    int frame_index;    // Renderer::frameIndex (1-based)
    int pad[3];
};

// Scene box of the Morton keys (min corner and extent per axis).
struct Box6 {
    float smin[3];
    float ssize[3];
};

// Morton keys written by the path-ray generation for the rays it creates
// (kind WFPT_MORTON_*; keys[i] and indices[i] = i per output ray i, as
// launch_morton writes them over the output rays).
struct MortonOut {
    int kind;
    void* keys;
    uint32_t* indices;
    Box6 box;
};

// Number of kernels this library has launched (all threads, all devices).
void count_launch(uint32_t k = 1);
uint64_t launch_count();

// Per-unit device status readers (return and clear).
cudaError_t status_stages(uint32_t* out);
cudaError_t status_sort(uint32_t* out);
cudaError_t status_trace(uint32_t* out);
// Failure-detection self-tests (one bounded device wait that cannot
// succeed; see sort.cu / stages.cu).
cudaError_t sort_selftest_timeout(cudaStream_t s);
cudaError_t raygen_path_selftest_timeout(cudaStream_t s);

cudaError_t launch_init_seeds(uint32_t* seeds, uint32_t n, int frame, cudaStream_t s,
                              const FrameParams* fp = nullptr);
cudaError_t launch_raygen_primary(const float* m, const int32_t* i2p, wfpt_ray* rays, const float* o,
                                  int sample_index, int w, int h, float max_dist, cudaStream_t s,
                                  const FrameParams* fp = nullptr, int pass = 0, int spp = 1);
cudaError_t launch_raygen_shadow(const uint32_t* seeds, const wfpt_ray* in_rays, const wfpt_hit* in_res,
                                 wfpt_ray* out_rays, int32_t* s2i, int32_t* i2s, const float* light,
                                 float radius, int bb, int bs, const uint32_t* n_in_dev, int S,
                                 cudaStream_t s);
size_t raygen_path_scratch_bytes(uint32_t max_n);
// mo (nullable): also the Morton keys of the output rays (what
// launch_morton over out_rays and *out_count would write).
cudaError_t launch_raygen_path(uint32_t* seeds, const wfpt_geometry* geoms, const wfpt_ray* in_rays,
                               wfpt_ray* out_rays, const int32_t* in_i2p, int32_t* out_i2p,
                               const wfpt_hit* in_res, float* decreases, uint32_t* out_count,
                               uint32_t n, const uint32_t* n_dev, float albedo, void* scratch,
                               cudaStream_t s, const MortonOut* mo = nullptr);
// launch_raygen_path over the library's static scratch (n at most
// WFPT_RAYGEN_PATH_STATIC_MAX_RAYS); calls on one device must not overlap.
cudaError_t launch_raygen_path_static(uint32_t* seeds, const wfpt_geometry* geoms, const wfpt_ray* in_rays,
                                      wfpt_ray* out_rays, const int32_t* in_i2p, int32_t* out_i2p,
                                      const wfpt_hit* in_res, float* decreases, uint32_t* out_count,
                                      uint32_t n, const uint32_t* n_dev, float albedo, cudaStream_t s);
cudaError_t launch_reconstruct_smooth(const wfpt_ray* rays, const wfpt_hit* res, const int32_t* i2p,
                                      float* pixels, const float* decreases, const wfpt_geometry* geoms,
                                      const float* light, const float* bg, uint32_t n,
                                      const uint32_t* n_dev, int spp, cudaStream_t s,
                                      uint32_t* hit_count = nullptr, bool fresh = false);
cudaError_t launch_reconstruct_shadow(const wfpt_hit* res, const int32_t* i2p, const int32_t* i2s,
                                      const float* in_pixels, float* out_pixels, int bb, int bs,
                                      const uint32_t* n_in_dev, int S, int replace, cudaStream_t s);
cudaError_t launch_count_hits(const wfpt_hit* res, uint32_t n, const uint32_t* n_dev, uint32_t* count,
                              cudaStream_t s);
cudaError_t launch_interpolate_colors(float* frame_pixels, float* pixels, uint32_t n, int frame_index,
                                      float key, float white, cudaStream_t s, const FrameParams* fp = nullptr);
cudaError_t launch_interpolate_colors_fp64(float* frame_pixels, float* pixels, double* accum, uint32_t n,
                                           int frame_index, float key, float white, cudaStream_t s,
                                           const FrameParams* fp = nullptr);
// Host-side one-time set-up that must not happen inside a stream capture
// (function attributes, occupancy queries).
// Every device or pinned-host allocation the library makes goes through
// these (cudaMalloc / cudaMallocHost); alloc_count() is the number made so
// far in this process (tuning key "debug.alloc_count").
cudaError_t dev_malloc(void** p, size_t bytes);
cudaError_t host_malloc(void** p, size_t bytes);
uint64_t alloc_count();
cudaError_t sort_prepare();
cudaError_t launch_fill_u32(void* dst, uint32_t v, size_t n, cudaStream_t s);
cudaError_t launch_batch_count(const uint32_t* n_in_dev, uint32_t begin, uint32_t size, int S, uint32_t* out,
                               cudaStream_t s);

// keys.cu
cudaError_t launch_morton(const wfpt_ray* rays, uint32_t n, const uint32_t* n_dev, const float* smin,
                          const float* ssize, int kind, void* keys, uint32_t* indices, cudaStream_t s);
cudaError_t launch_reorder(const uint32_t* idx, const wfpt_ray* in_rays, wfpt_ray* out_rays,
                           const int32_t* in_s2i, int32_t* out_s2i, int32_t* out_i2s, uint32_t n,
                           const uint32_t* n_dev, cudaStream_t s);
// record_bytes 16, 32, 48 or 64; slot maps optional (all three or none).
cudaError_t launch_reorder_records(const uint32_t* idx, const void* in_records, void* out_records,
                                   uint32_t record_bytes, const int32_t* in_s2i, int32_t* out_s2i, int32_t* out_i2s,
                                   uint32_t n, const uint32_t* n_dev, cudaStream_t s);

// sort.cu
size_t sort_scratch_bytes(uint32_t max_n, int key_bits);
// Sort tile variant: 0 = automatic by size, 1 = small tiles, 2 = large tiles.
void set_sort_tiles(int v);
int get_sort_tiles();
// Radix digit width: 8 (default) or 4 bits per pass.
void set_sort_digit_bits(int v);
int get_sort_digit_bits();
cudaError_t launch_sort_pairs(void* keys, uint32_t* values, uint32_t n, const uint32_t* n_dev,
                              int key_bits, void* scratch, size_t scratch_bytes, cudaStream_t s);

}  // namespace wfpt
