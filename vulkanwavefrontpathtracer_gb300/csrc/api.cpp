// C ABI of libwfpt: argument checks, CUDA error mapping and the scene
// object.  Every stage entry point validates its arguments on the host and
// forwards to one launcher; nothing here falls back to host computation.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/wfpt.h"
#include "build.cuh"
#include "host.h"
#include "internal.h"
#include "scene.h"
#include "stages.cuh"
#include "trace.cuh"

namespace {

thread_local std::string g_last_error;

wfpt_status invalid(const char* what) {
    g_last_error = what;
    return WFPT_ERR_INVALID_ARGUMENT;
}

}  // namespace

namespace wfpt {

wfpt_status from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return WFPT_OK;
    g_last_error = cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? WFPT_ERR_OUT_OF_MEMORY : WFPT_ERR_CUDA;
}

void set_error(const char* msg) { g_last_error = msg; }

}  // namespace wfpt

using wfpt::from_cuda;

struct wfpt_scene {
    wfpt::HostBvh2 bvh2;  // plain-form BVH kept on the host for export
    wfpt::HostBvh8 bvh8;
    wfpt::SceneDevice dev;
    void* bufs[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    wfpt_scene_info info{};
    bool has2 = false, has8 = false, host_only = false;
    bool device_built = false;  // BVHs built on the GPU: no host copies
    uint32_t dev_bvh2_count = 0, dev_bvh8_count = 0, dev_ntris = 0;
};

namespace wfpt {
const SceneDevice* scene_device(const wfpt_scene* s) { return &s->dev; }
bool scene_has(const wfpt_scene* s, int kind) {
    return !s->host_only && (kind == WFPT_BVH8_Q8 ? s->has8 : s->has2);
}
void scene_bounds(const wfpt_scene* s, float mn[3], float mx[3]) {
    for (int k = 0; k < 3; ++k) {
        mn[k] = s->info.bounds_min[k];
        mx[k] = s->info.bounds_max[k];
    }
}
}  // namespace wfpt

extern "C" {

int wfpt_abi_version(void) { return WFPT_ABI_VERSION; }

const char* wfpt_status_string(wfpt_status s) {
    switch (s) {
        case WFPT_OK: return "ok";
        case WFPT_ERR_INVALID_ARGUMENT: return "invalid argument";
        case WFPT_ERR_CUDA: return "CUDA error";
        case WFPT_ERR_OUT_OF_MEMORY: return "out of memory";
        case WFPT_ERR_TIMEOUT: return "device wait timed out";
        case WFPT_ERR_UNSUPPORTED: return "unsupported";
        case WFPT_ERR_SCRATCH_TOO_SMALL: return "scratch too small";
        case WFPT_ERR_DEVICE_BOUNDS: return "device bounds check fired";
    }
    return "unknown status";
}

const char* wfpt_last_error_message(void) { return g_last_error.c_str(); }

uint64_t wfpt_kernel_launch_count(void) { return wfpt::launch_count(); }

wfpt_status wfpt_tune_set(const char* key, int64_t value) {
    if (!key) return invalid("null key");
    std::string k(key);
    if (k == "trace.bvh8.refill") {
        if (value < 1 || value > 32) return invalid("trace.bvh8.refill must be in [1, 32]");
        wfpt::set_trace_refill((uint32_t)value);
        return WFPT_OK;
    }
    if (k == "trace.bvh8.postpone") {
        if (value < 0 || value > 32) return invalid("trace.bvh8.postpone must be in [0, 32]");
        wfpt::set_trace_postpone((uint32_t)value);
        return WFPT_OK;
    }
    if (k == "trace.bvh8.batch" || k == "trace.bvh8.any_batch") {
        if (value < 1 || value > 32) return invalid((k + " must be in [1, 32]").c_str());
        wfpt::set_trace_batch((uint32_t)value, k == "trace.bvh8.batch");
        return WFPT_OK;
    }
    if (k == "trace.bvh8.steps" || k == "trace.bvh8.any_steps") {
        if (value < 1 || value > 8) return invalid((k + " must be in [1, 8]").c_str());
        wfpt::set_trace_steps((uint32_t)value, k == "trace.bvh8.steps");
        return WFPT_OK;
    }
    if (k == "trace.bvh8.coop") {
        if (value < 0 || value > 1) return invalid("trace.bvh8.coop must be 0 or 1");
        wfpt::set_trace_coop(value != 0);
        return WFPT_OK;
    }
    if (k == "sort.tiles") {
        if (value < 0 || value > 3)
            return invalid("sort.tiles must be 0 (auto), 1 (small), 2 (large) or 3 (extra-large)");
        wfpt::set_sort_tiles((int)value);
        return WFPT_OK;
    }
    if (k == "sort.digit_bits") {
        if (value != 4 && value != 8) return invalid("sort.digit_bits must be 4 or 8");
        wfpt::set_sort_digit_bits((int)value);
        return WFPT_OK;
    }
    if (k == "debug.alloc_count") return invalid("debug.alloc_count is read-only");
    if (k == "debug.fail_alloc_after") {
        if (value < -1 || value > (1 << 20)) return invalid("debug.fail_alloc_after must be in [-1, 2^20]");
        wfpt::set_fail_alloc_after((int)value);
        return WFPT_OK;
    }
    if (k == "renderer.shadow_slots") {
        if (value < 0 || value > 8) return invalid("renderer.shadow_slots must be 0 (planned) or in [1, 8]");
        wfpt::set_shadow_slots((int)value);
        return WFPT_OK;
    }
    if (k == "build.ploc.radius") {
        if (value < 1 || value > 64) return invalid("build.ploc.radius must be in [1, 64]");
        wfpt::set_ploc_radius((int)value);
        return WFPT_OK;
    }
    if (k == "build.bvh8.collapse") {
        if (value < 0 || value > 1) return invalid("build.bvh8.collapse must be 0 (greedy) or 1 (SAH)");
        wfpt::set_bvh8_collapse((int)value);
        return WFPT_OK;
    }
    if (k == "build.bvh8.tri_cost") {
        if (value < 1 || value > 10000) return invalid("build.bvh8.tri_cost must be in [1, 10000] percent");
        wfpt::set_bvh8_tri_cost_pct((int)value);
        return WFPT_OK;
    }
    if (k == "trace.count") {
        if (value < 0 || value > 1) return invalid("trace.count must be 0 or 1");
        wfpt::set_trace_count(value != 0);
        return WFPT_OK;
    }
    return invalid("unknown tuning key");
}

wfpt_status wfpt_trace_counters(uint64_t out[4], int reset) {
    if (!out) return invalid("null output");
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = wfpt::trace_counters(out, reset != 0);
    return from_cuda(e);
}

wfpt_status wfpt_tune_get(const char* key, int64_t* value) {
    if (!key || !value) return invalid("null argument");
    std::string k(key);
    if (k == "trace.bvh8.refill") {
        *value = wfpt::get_trace_refill();
        return WFPT_OK;
    }
    if (k == "trace.bvh8.postpone") {
        *value = wfpt::get_trace_postpone();
        return WFPT_OK;
    }
    if (k == "trace.bvh8.batch" || k == "trace.bvh8.any_batch") {
        *value = (int64_t)wfpt::get_trace_batch(k == "trace.bvh8.batch");
        return WFPT_OK;
    }
    if (k == "trace.bvh8.steps" || k == "trace.bvh8.any_steps") {
        *value = (int64_t)wfpt::get_trace_steps(k == "trace.bvh8.steps");
        return WFPT_OK;
    }
    if (k == "trace.bvh8.coop") {
        *value = wfpt::get_trace_coop() ? 1 : 0;
        return WFPT_OK;
    }
    if (k == "sort.tiles") {
        *value = wfpt::get_sort_tiles();
        return WFPT_OK;
    }
    if (k == "sort.digit_bits") {
        *value = wfpt::get_sort_digit_bits();
        return WFPT_OK;
    }
    if (k == "debug.alloc_count") {
        *value = (int64_t)wfpt::alloc_count();
        return WFPT_OK;
    }
    if (k == "debug.fail_alloc_after") {
        *value = wfpt::get_fail_alloc_after();
        return WFPT_OK;
    }
    if (k == "renderer.shadow_slots") {
        *value = wfpt::get_shadow_slots();
        return WFPT_OK;
    }
    if (k == "build.ploc.radius") {
        *value = wfpt::get_ploc_radius();
        return WFPT_OK;
    }
    if (k == "build.bvh8.collapse") {
        *value = wfpt::get_bvh8_collapse();
        return WFPT_OK;
    }
    if (k == "build.bvh8.tri_cost") {
        *value = wfpt::get_bvh8_tri_cost_pct();
        return WFPT_OK;
    }
    if (k == "trace.count") {
        *value = wfpt::get_trace_count() ? 1 : 0;
        return WFPT_OK;
    }
    return invalid("unknown tuning key");
}

wfpt_status wfpt_device_status(uint32_t* flags) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return from_cuda(e);
    uint32_t v = 0;
    if ((e = wfpt::status_stages(&v)) != cudaSuccess) return from_cuda(e);
    if ((e = wfpt::status_sort(&v)) != cudaSuccess) return from_cuda(e);
    if ((e = wfpt::status_trace(&v)) != cudaSuccess) return from_cuda(e);
    if ((e = wfpt::status_build(&v)) != cudaSuccess) return from_cuda(e);
    if (flags) *flags = v;
    if (v & wfpt::kStatusTimeout) {
        g_last_error = "a bounded device-side wait gave up";
        return WFPT_ERR_TIMEOUT;
    }
    if (v & wfpt::kStatusBounds) {
        g_last_error = "a device-side bounds check fired";
        return WFPT_ERR_DEVICE_BOUNDS;
    }
    return WFPT_OK;
}

wfpt_status wfpt_selftest_wait_timeout(int which) {
    if (which != 0 && which != 1) return invalid("which must be 0 (radix sort) or 1 (path compaction)");
    cudaError_t e = cudaDeviceSynchronize();
    uint32_t before = 0;
    if (e == cudaSuccess) e = wfpt::status_stages(&before);
    if (e == cudaSuccess) e = wfpt::status_sort(&before);
    if (e != cudaSuccess) return from_cuda(e);
    if (before) {
        g_last_error = "device status was already set before the self-test";
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    e = which == 0 ? wfpt::sort_selftest_timeout(nullptr) : wfpt::raygen_path_selftest_timeout(nullptr);
    if (e != cudaSuccess) return from_cuda(e);
    return wfpt_device_status(nullptr);
}

wfpt_status wfpt_pixel_table(int width, int height, int32_t* index_to_pixel, int32_t* pixel_to_index) {
    if (width <= 0 || height <= 0) return invalid("width and height must be positive");
    if ((long long)width * height > (1ll << 30)) return invalid("image too large");
    if (!index_to_pixel || !pixel_to_index) return invalid("null output buffer");
    wfpt::pixel_table(width, height, index_to_pixel, pixel_to_index);
    return WFPT_OK;
}

wfpt_status wfpt_camera_screen_to_world(const float position[3], const float rotation_deg[3], float fov_deg,
                                        float aspect, float znear, float zfar, float screen_to_world[16]) {
    if (!position || !rotation_deg || !screen_to_world) return invalid("null pointer");
    if (!(fov_deg > 0.0f && fov_deg < 180.0f)) return invalid("fov must be in (0, 180)");
    if (!(aspect > 0.0f) || !(znear > 0.0f) || !(zfar > znear)) return invalid("bad projection parameters");
    if (!wfpt::camera_screen_to_world(position, rotation_deg, fov_deg, aspect, znear, zfar, screen_to_world))
        return invalid("singular camera matrix");
    return WFPT_OK;
}

// ------------------------------------------------------------ stages
#define WFPT_REQUIRE(cond, msg) \
    do {                        \
        if (!(cond)) return invalid(msg); \
    } while (0)

static inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }
static constexpr uint32_t kMaxN = (1u << 30) - 1u;

wfpt_status wfpt_init_seeds(uint32_t* seeds, uint32_t n, int frame_index, void* stream) {
    WFPT_REQUIRE(n == 0 || seeds, "seeds is null");
    return from_cuda(wfpt::launch_init_seeds(seeds, n, frame_index, S(stream)));
}

wfpt_status wfpt_raygen_primary(const float screen_to_world[16], const int32_t* index_to_pixel, wfpt_ray* rays,
                                const float origin[3], int sample_index, int width, int height, float max_dist,
                                void* stream) {
    WFPT_REQUIRE(screen_to_world && origin, "null matrix or origin");
    WFPT_REQUIRE(width >= 0 && height >= 0, "negative size");
    WFPT_REQUIRE((long long)width * height <= kMaxN, "image too large");
    WFPT_REQUIRE(sample_index >= 0, "negative sample index");
    WFPT_REQUIRE((long long)width * height == 0 || (index_to_pixel && rays), "null buffer");
    return from_cuda(wfpt::launch_raygen_primary(screen_to_world, index_to_pixel, rays, origin, sample_index, width,
                                                 height, max_dist, S(stream)));
}

wfpt_status wfpt_morton(const wfpt_ray* rays, uint32_t n, const uint32_t* n_dev, const float scene_min[3],
                        const float scene_size[3], int morton_kind, void* keys, uint32_t* indices, void* stream) {
    WFPT_REQUIRE(n <= kMaxN, "n too large");
    WFPT_REQUIRE(scene_min && scene_size, "null scene box");
    WFPT_REQUIRE(morton_kind >= WFPT_MORTON_AILA32 && morton_kind <= WFPT_MORTON_6D64, "unknown morton kind");
    WFPT_REQUIRE(n == 0 || (rays && keys && indices), "null buffer");
    return from_cuda(wfpt::launch_morton(rays, n, n_dev, scene_min, scene_size, morton_kind, keys, indices,
                                         S(stream)));
}

size_t wfpt_sort_scratch_bytes(uint32_t max_n, int key_bits) { return wfpt::sort_scratch_bytes(max_n, key_bits); }

wfpt_status wfpt_sort_pairs(void* keys, uint32_t* values, uint32_t n, const uint32_t* n_dev, int key_bits,
                            void* scratch, size_t scratch_bytes, void* stream) {
    WFPT_REQUIRE(key_bits >= 1 && key_bits <= 64, "key_bits must be in [1, 64]");
    WFPT_REQUIRE(n <= kMaxN, "n too large");
    if (n == 0) return WFPT_OK;
    WFPT_REQUIRE(keys && values && scratch, "null buffer");
    if (scratch_bytes < wfpt::sort_scratch_bytes(n, key_bits)) {
        g_last_error = "sort scratch smaller than wfpt_sort_scratch_bytes(n, key_bits)";
        return WFPT_ERR_SCRATCH_TOO_SMALL;
    }
    return from_cuda(wfpt::launch_sort_pairs(keys, values, n, n_dev, key_bits, scratch, scratch_bytes, S(stream)));
}

wfpt_status wfpt_reorder(const uint32_t* ray_index, const wfpt_ray* in_rays, wfpt_ray* out_rays,
                         const int32_t* in_slot_to_index, int32_t* out_slot_to_index, int32_t* out_index_to_slot,
                         uint32_t n, const uint32_t* n_dev, void* stream) {
    WFPT_REQUIRE(n <= kMaxN, "n too large");
    WFPT_REQUIRE(n == 0 || (ray_index && in_rays && out_rays && in_slot_to_index && out_slot_to_index &&
                            out_index_to_slot),
                 "null buffer");
    WFPT_REQUIRE(n == 0 || (const void*)in_rays != (const void*)out_rays, "reorder cannot run in place");
    return from_cuda(wfpt::launch_reorder(ray_index, in_rays, out_rays, in_slot_to_index, out_slot_to_index,
                                          out_index_to_slot, n, n_dev, S(stream)));
}

wfpt_status wfpt_reorder_records(const uint32_t* ray_index, const void* in_records, void* out_records,
                                 uint32_t record_bytes, const int32_t* in_slot_to_index, int32_t* out_slot_to_index,
                                 int32_t* out_index_to_slot, uint32_t n, const uint32_t* n_dev, void* stream) {
    WFPT_REQUIRE(n <= kMaxN, "n too large");
    WFPT_REQUIRE(record_bytes == 16 || record_bytes == 32 || record_bytes == 48 || record_bytes == 64,
                 "record_bytes must be 16, 32, 48 or 64");
    const bool maps = in_slot_to_index || out_slot_to_index || out_index_to_slot;
    WFPT_REQUIRE(!maps || (in_slot_to_index && out_slot_to_index && out_index_to_slot),
                 "slot maps: pass all three or none");
    WFPT_REQUIRE(n == 0 || (ray_index && in_records && out_records), "null buffer");
    WFPT_REQUIRE(n == 0 || ((reinterpret_cast<uintptr_t>(in_records) | reinterpret_cast<uintptr_t>(out_records)) &
                            15u) == 0,
                 "record buffers must be 16-byte aligned");
    WFPT_REQUIRE(n == 0 || in_records != (const void*)out_records, "reorder cannot run in place");
    return from_cuda(wfpt::launch_reorder_records(ray_index, in_records, out_records, record_bytes, in_slot_to_index,
                                                  out_slot_to_index, out_index_to_slot, n, n_dev, S(stream)));
}

wfpt_status wfpt_raygen_shadow(const uint32_t* seeds, const wfpt_ray* in_rays, const wfpt_hit* in_results,
                               wfpt_ray* out_rays, int32_t* out_slot_to_index, int32_t* out_index_to_slot,
                               const float light[3], float light_radius, int batch_begin, int batch_size,
                               const uint32_t* n_in_dev, int num_samples, void* stream) {
    WFPT_REQUIRE(light, "null light");
    WFPT_REQUIRE(batch_begin >= 0 && batch_size >= 0, "negative batch");
    WFPT_REQUIRE(num_samples >= 1 && num_samples <= 1024, "num_samples must be in [1, 1024]");
    WFPT_REQUIRE((long long)batch_size * num_samples <= kMaxN, "batch too large");
    WFPT_REQUIRE(batch_size == 0 || (seeds && in_rays && in_results && out_rays && out_slot_to_index &&
                                     out_index_to_slot),
                 "null buffer");
    return from_cuda(wfpt::launch_raygen_shadow(seeds, in_rays, in_results, out_rays, out_slot_to_index,
                                                out_index_to_slot, light, light_radius, batch_begin, batch_size,
                                                n_in_dev, num_samples, S(stream)));
}

size_t wfpt_raygen_path_scratch_bytes(uint32_t max_n) { return wfpt::raygen_path_scratch_bytes(max_n); }

wfpt_status wfpt_raygen_path(uint32_t* seeds, const wfpt_geometry* geometries, const wfpt_ray* in_rays,
                             wfpt_ray* out_rays, const int32_t* in_index_to_pixel, int32_t* out_index_to_pixel,
                             const wfpt_hit* in_results, float* decreases, uint32_t* out_count_dev, uint32_t n,
                             const uint32_t* n_dev, int russian_roulette, float albedo, void* scratch,
                             size_t scratch_bytes, void* stream) {
    (void)russian_roulette;  // read but unused by the reference shader (raygenPath.comp:73)
    WFPT_REQUIRE(n <= kMaxN, "n too large");
    WFPT_REQUIRE(out_count_dev && scratch, "null counter or scratch");
    WFPT_REQUIRE(n == 0 || (seeds && geometries && in_rays && out_rays && in_index_to_pixel && out_index_to_pixel &&
                            in_results && decreases),
                 "null buffer");
    if (scratch_bytes < wfpt::raygen_path_scratch_bytes(n)) {
        g_last_error = "path scratch smaller than wfpt_raygen_path_scratch_bytes(n)";
        return WFPT_ERR_SCRATCH_TOO_SMALL;
    }
    return from_cuda(wfpt::launch_raygen_path(seeds, geometries, in_rays, out_rays, in_index_to_pixel,
                                              out_index_to_pixel, in_results, decreases, out_count_dev, n, n_dev,
                                              albedo, scratch, S(stream)));
}

wfpt_status wfpt_raygen_path_static(uint32_t* seeds, const wfpt_geometry* geometries, const wfpt_ray* in_rays,
                                    wfpt_ray* out_rays, const int32_t* in_index_to_pixel,
                                    int32_t* out_index_to_pixel, const wfpt_hit* in_results, float* decreases,
                                    uint32_t* out_count_dev, uint32_t n, const uint32_t* n_dev,
                                    int russian_roulette, float albedo, void* stream) {
    (void)russian_roulette;
    WFPT_REQUIRE(n <= WFPT_RAYGEN_PATH_STATIC_MAX_RAYS,
                 "n exceeds WFPT_RAYGEN_PATH_STATIC_MAX_RAYS (16777216); use wfpt_raygen_path with caller scratch");
    WFPT_REQUIRE(out_count_dev, "null counter");
    WFPT_REQUIRE(n == 0 || (seeds && geometries && in_rays && out_rays && in_index_to_pixel && out_index_to_pixel &&
                            in_results && decreases),
                 "null buffer");
    cudaError_t e = wfpt::launch_raygen_path_static(seeds, geometries, in_rays, out_rays, in_index_to_pixel,
                                                    out_index_to_pixel, in_results, decreases, out_count_dev, n,
                                                    n_dev, albedo, S(stream));
    if (e == cudaErrorStreamCaptureUnsupported)
        return invalid("first wfpt_raygen_path_static call in this CUDA context made while the stream is capturing; "
                       "make one call outside any stream capture first (it looks up the scratch array's address)");
    return from_cuda(e);
}

wfpt_status wfpt_reconstruct_smooth(const wfpt_ray* rays, const wfpt_hit* results, const int32_t* index_to_pixel,
                                    float* pixels, const float* decreases, const wfpt_geometry* geometries,
                                    const float light[3], const float background[3], uint32_t n,
                                    const uint32_t* n_dev, int num_samples, void* stream) {
    WFPT_REQUIRE(light && background, "null light or background");
    WFPT_REQUIRE(num_samples >= 1, "num_samples must be positive");
    WFPT_REQUIRE(n <= kMaxN, "n too large");
    WFPT_REQUIRE(n == 0 || (rays && results && index_to_pixel && pixels && decreases && geometries), "null buffer");
    return from_cuda(wfpt::launch_reconstruct_smooth(rays, results, index_to_pixel, pixels, decreases, geometries,
                                                     light, background, n, n_dev, num_samples, S(stream)));
}

wfpt_status wfpt_reconstruct_shadow(const wfpt_hit* shadow_results, const int32_t* index_to_pixel,
                                    const int32_t* index_to_slot, const float* in_pixels, float* out_pixels,
                                    int batch_begin, int batch_size, const uint32_t* n_in_dev, int num_samples,
                                    int replace, void* stream) {
    WFPT_REQUIRE(batch_begin >= 0 && batch_size >= 0, "negative batch");
    WFPT_REQUIRE(num_samples >= 1 && num_samples <= 1024, "num_samples must be in [1, 1024]");
    WFPT_REQUIRE(batch_size == 0 || (shadow_results && index_to_pixel && index_to_slot && in_pixels && out_pixels),
                 "null buffer");
    return from_cuda(wfpt::launch_reconstruct_shadow(shadow_results, index_to_pixel, index_to_slot, in_pixels,
                                                     out_pixels, batch_begin, batch_size, n_in_dev, num_samples,
                                                     replace, S(stream)));
}

wfpt_status wfpt_count_hits(const wfpt_hit* results, uint32_t n, const uint32_t* n_dev, uint32_t* count_dev,
                            void* stream) {
    WFPT_REQUIRE(count_dev, "null counter");
    WFPT_REQUIRE(n <= kMaxN, "n too large");
    WFPT_REQUIRE(n == 0 || results, "null results");
    return from_cuda(wfpt::launch_count_hits(results, n, n_dev, count_dev, S(stream)));
}

wfpt_status wfpt_interpolate_colors(float* frame_pixels, float* pixels, uint32_t num_pixels, int frame_index,
                                    float key_value, float white_point, void* stream) {
    WFPT_REQUIRE(num_pixels <= kMaxN, "too many pixels");
    WFPT_REQUIRE(num_pixels == 0 || (frame_pixels && pixels), "null buffer");
    return from_cuda(
        wfpt::launch_interpolate_colors(frame_pixels, pixels, num_pixels, frame_index, key_value, white_point, S(stream)));
}

wfpt_status wfpt_interpolate_colors_fp64(float* frame_pixels, float* pixels, double* accum, uint32_t num_pixels,
                                         int frame_index, float key_value, float white_point, void* stream) {
    WFPT_REQUIRE(num_pixels <= kMaxN, "too many pixels");
    WFPT_REQUIRE(num_pixels == 0 || (frame_pixels && pixels && accum), "null buffer");
    WFPT_REQUIRE(reinterpret_cast<uintptr_t>(accum) % 32 == 0, "accum must be 32-byte aligned");
    return from_cuda(wfpt::launch_interpolate_colors_fp64(frame_pixels, pixels, accum, num_pixels, frame_index,
                                                          key_value, white_point, S(stream)));
}

wfpt_status wfpt_fill_u32(void* dst, uint32_t pattern, size_t count_u32, void* stream) {
    WFPT_REQUIRE(count_u32 == 0 || dst, "null buffer");
    return from_cuda(wfpt::launch_fill_u32(dst, pattern, count_u32, S(stream)));
}

// ------------------------------------------------------------- scene
static cudaError_t upload(void** dst, const void* src, size_t bytes) {
    cudaError_t e = wfpt::dev_malloc(dst, bytes);
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
}

static wfpt_status check_geometry_table(const uint32_t* geometry_first_triangle, uint32_t num_geometries,
                                        uint32_t num_triangles) {
    if (geometry_first_triangle && num_geometries > 0) {
        WFPT_REQUIRE(geometry_first_triangle[0] == 0, "geometry_first_triangle[0] must be 0");
        for (uint32_t g = 1; g < num_geometries; ++g)
            WFPT_REQUIRE(geometry_first_triangle[g] >= geometry_first_triangle[g - 1] &&
                             geometry_first_triangle[g] <= num_triangles,
                         "geometry_first_triangle must ascend within [0, num_triangles]");
    }
    return WFPT_OK;
}

// A scene whose BVHs are built on the device from device-resident geometry
// (at least two triangles; build.cu).
static wfpt_status create_device_built(const float* positions_dev, uint32_t num_vertices,
                                       const uint32_t* indices_dev, uint32_t num_triangles,
                                       const uint32_t* geometry_first_triangle, uint32_t num_geometries,
                                       int bvh_kinds_mask, cudaStream_t s,
                                       std::chrono::steady_clock::time_point t0, wfpt_scene** scene) {
    std::vector<uint32_t> gf(num_geometries ? num_geometries : 1u, 0u);
    if (geometry_first_triangle && num_geometries)
        std::memcpy(gf.data(), geometry_first_triangle, gf.size() * sizeof(uint32_t));
    void* gdev = nullptr;
    cudaError_t e = upload(&gdev, gf.data(), gf.size() * sizeof(uint32_t));
    if (e != cudaSuccess) return from_cuda(e);
    wfpt::DeviceBuild b;
    e = wfpt::build_scene_device(positions_dev, num_vertices, indices_dev, num_triangles,
                                 reinterpret_cast<const uint32_t*>(gdev), (uint32_t)gf.size(),
                                 (bvh_kinds_mask & (1 << WFPT_BVH8_Q8)) != 0, s, &b);
    cudaFree(gdev);
    if (e == cudaErrorInvalidValue) return invalid("triangle index out of range");
    if (e != cudaSuccess) {
        wfpt_status st = from_cuda(e);
        g_last_error = std::string("device BVH build failed: ") + g_last_error;
        return st;
    }
    wfpt_scene* sc = new (std::nothrow) wfpt_scene();
    if (!sc) {
        for (void* p : {b.bvh2_nodes, b.bvh2_tris, b.bvh8_nodes, b.bvh8_tris})
            if (p) cudaFree(p);
        return WFPT_ERR_OUT_OF_MEMORY;
    }
    sc->device_built = true;
    sc->has2 = (bvh_kinds_mask & (1 << WFPT_BVH2_FP32)) != 0;
    sc->has8 = (bvh_kinds_mask & (1 << WFPT_BVH8_Q8)) != 0;
    if (sc->has2) {
        sc->bufs[0] = b.bvh2_nodes;
        sc->bufs[1] = b.bvh2_tris;
    } else {
        cudaFree(b.bvh2_nodes);
        cudaFree(b.bvh2_tris);
    }
    sc->bufs[2] = b.bvh8_nodes;
    sc->bufs[3] = b.bvh8_tris;
    e = wfpt::dev_malloc(&sc->bufs[4], wfpt::kWorkSlots * 16 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(sc->bufs[4], 0, wfpt::kWorkSlots * 16 * sizeof(uint32_t));
    if (e != cudaSuccess) {
        wfpt_scene_destroy(sc);
        return from_cuda(e);
    }
    sc->dev.work = reinterpret_cast<uint32_t*>(sc->bufs[4]);
    sc->dev.bvh2_nodes = reinterpret_cast<const float4*>(sc->bufs[0]);
    sc->dev.bvh2_tris = reinterpret_cast<const float4*>(sc->bufs[1]);
    sc->dev.bvh8_nodes = reinterpret_cast<const float4*>(sc->bufs[2]);
    sc->dev.bvh8_tris = reinterpret_cast<const float4*>(sc->bufs[3]);
    sc->dev.bvh8_num_tris = sc->has8 ? num_triangles : 0u;
    sc->dev_bvh2_count = sc->has2 ? b.bvh2_count : 0u;
    sc->dev_bvh8_count = sc->has8 ? b.bvh8_count : 0u;
    sc->dev_ntris = num_triangles;
    sc->info.num_triangles = num_triangles;
    sc->info.num_geometries = (uint32_t)gf.size();
    sc->info.bvh2_nodes = sc->dev_bvh2_count;
    sc->info.bvh8_nodes = sc->dev_bvh8_count;
    for (int k = 0; k < 3; ++k) {
        sc->info.bounds_min[k] = b.bounds_min[k];
        sc->info.bounds_max[k] = b.bounds_max[k];
    }
    sc->info.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    *scene = sc;
    return WFPT_OK;
}

wfpt_status wfpt_scene_create_device(const float* positions_dev, uint32_t num_vertices,
                                     const uint32_t* indices_dev, uint32_t num_triangles,
                                     const uint32_t* geometry_first_triangle, uint32_t num_geometries,
                                     int bvh_kinds_mask, void* stream, wfpt_scene** scene) {
    WFPT_REQUIRE(scene, "null scene out-pointer");
    *scene = nullptr;
    WFPT_REQUIRE(num_triangles == 0 || (positions_dev && indices_dev), "null mesh");
    WFPT_REQUIRE(num_triangles < (1u << 27), "too many triangles (max 2^27 - 1)");
    WFPT_REQUIRE((bvh_kinds_mask & 3) != 0, "bvh_kinds_mask selects no BVH");
    WFPT_REQUIRE((bvh_kinds_mask & WFPT_SCENE_HOST_ONLY) == 0, "a device-built scene cannot be host-only");
    WFPT_REQUIRE(num_triangles == 0 || num_vertices > 0, "triangles without vertices");
    wfpt_status st = check_geometry_table(geometry_first_triangle, num_geometries, num_triangles);
    if (st != WFPT_OK) return st;
    auto t0 = std::chrono::steady_clock::now();
    if (num_triangles < 2) {
        // One triangle or none: the host builder's wrapped or empty root.
        std::vector<uint32_t> idx(3ull * num_triangles);
        std::vector<float> pos(3ull * num_vertices);
        cudaError_t e = cudaSuccess;
        if (!idx.empty()) e = cudaMemcpy(idx.data(), indices_dev, idx.size() * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && !pos.empty())
            e = cudaMemcpy(pos.data(), positions_dev, pos.size() * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return from_cuda(e);
        return wfpt_scene_create(pos.data(), num_vertices, idx.data(), num_triangles, geometry_first_triangle,
                                 num_geometries, bvh_kinds_mask & 3, scene);
    }
    return create_device_built(positions_dev, num_vertices, indices_dev, num_triangles, geometry_first_triangle,
                               num_geometries, bvh_kinds_mask & 3, S(stream), t0, scene);
}

wfpt_status wfpt_scene_create(const float* positions, uint32_t num_vertices, const uint32_t* indices,
                              uint32_t num_triangles, const uint32_t* geometry_first_triangle,
                              uint32_t num_geometries, int bvh_kinds_mask, wfpt_scene** scene) {
    WFPT_REQUIRE(scene, "null scene out-pointer");
    *scene = nullptr;
    WFPT_REQUIRE(num_triangles == 0 || (positions && indices), "null mesh");
    WFPT_REQUIRE(num_triangles < (1u << 27), "too many triangles (max 2^27 - 1)");
    WFPT_REQUIRE((bvh_kinds_mask & 3) != 0, "bvh_kinds_mask selects no BVH");
    WFPT_REQUIRE((bvh_kinds_mask & WFPT_SCENE_HOST_ONLY) == 0 || (bvh_kinds_mask & WFPT_SCENE_DEVICE_BUILD) == 0,
                 "a device-built scene cannot be host-only");
    for (uint64_t i = 0; i < 3ull * num_triangles; ++i)
        if (indices[i] >= num_vertices) return invalid("triangle index out of range");
    wfpt_status gst = check_geometry_table(geometry_first_triangle, num_geometries, num_triangles);
    if (gst != WFPT_OK) return gst;
    auto t0 = std::chrono::steady_clock::now();
    if ((bvh_kinds_mask & WFPT_SCENE_DEVICE_BUILD) && num_triangles >= 2) {
        void* pd = nullptr;
        void* id = nullptr;
        cudaError_t e = upload(&pd, positions, 3ull * num_vertices * sizeof(float));
        if (e == cudaSuccess) e = upload(&id, indices, 3ull * num_triangles * sizeof(uint32_t));
        wfpt_status st = e == cudaSuccess ? WFPT_OK : from_cuda(e);
        if (st == WFPT_OK)
            st = create_device_built(reinterpret_cast<const float*>(pd), num_vertices,
                                     reinterpret_cast<const uint32_t*>(id), num_triangles, geometry_first_triangle,
                                     num_geometries, bvh_kinds_mask & 3, nullptr, t0, scene);
        if (pd) cudaFree(pd);
        if (id) cudaFree(id);
        return st;
    }
    wfpt_scene* sc = new (std::nothrow) wfpt_scene();
    if (!sc) return WFPT_ERR_OUT_OF_MEMORY;
    wfpt::BuildInput in{positions, num_vertices, indices, num_triangles, geometry_first_triangle,
                        num_geometries == 0 ? 1u : num_geometries};
    try {
        wfpt::HostBvh2 for8;
        if (bvh_kinds_mask & (1 << WFPT_BVH2_FP32)) {
            wfpt::build_bvh2(in, 4, sc->bvh2);
            sc->has2 = true;
        }
        wfpt::HostBvh8& b8 = sc->bvh8;
        if (bvh_kinds_mask & (1 << WFPT_BVH8_Q8)) {
            wfpt::build_bvh2(in, 1, for8);  // single-triangle leaves: the collapse decides leaf sizes
            wfpt::build_bvh8(for8, b8);
            sc->has8 = true;
            if (!sc->has2) sc->bvh2 = for8;
        }
        sc->host_only = (bvh_kinds_mask & WFPT_SCENE_HOST_ONLY) != 0;
        cudaError_t e = cudaSuccess;
        if (sc->host_only) {
            // no upload
        } else if (sc->has2) {
            e = upload(&sc->bufs[0], sc->bvh2.nodes.data(), sc->bvh2.nodes.size() * sizeof(wfpt::Bvh2Node));
            if (e == cudaSuccess)
                e = upload(&sc->bufs[1], sc->bvh2.tris.data(), sc->bvh2.tris.size() * sizeof(wfpt::TriRec));
        }
        if (e == cudaSuccess && sc->has8 && !sc->host_only) {
            e = upload(&sc->bufs[2], b8.nodes.data(), b8.nodes.size() * sizeof(wfpt::Bvh8Node));
            if (e == cudaSuccess) e = upload(&sc->bufs[3], b8.tris.data(), b8.tris.size() * sizeof(wfpt::TriRec));
            sc->dev.bvh8_num_tris = (uint32_t)b8.tris.size();
        }
        if (e == cudaSuccess && !sc->host_only) {
            e = wfpt::dev_malloc(&sc->bufs[4], wfpt::kWorkSlots * 16 * sizeof(uint32_t));
            if (e == cudaSuccess) e = cudaMemset(sc->bufs[4], 0, wfpt::kWorkSlots * 16 * sizeof(uint32_t));
            sc->dev.work = reinterpret_cast<uint32_t*>(sc->bufs[4]);
        }
        if (e != cudaSuccess) {
            wfpt_scene_destroy(sc);
            return from_cuda(e);
        }
        sc->dev.bvh2_nodes = reinterpret_cast<const float4*>(sc->bufs[0]);
        sc->dev.bvh2_tris = reinterpret_cast<const float4*>(sc->bufs[1]);
        sc->dev.bvh8_nodes = reinterpret_cast<const float4*>(sc->bufs[2]);
        sc->dev.bvh8_tris = reinterpret_cast<const float4*>(sc->bufs[3]);
        sc->info.num_triangles = num_triangles;
        sc->info.num_geometries = num_geometries == 0 ? 1 : num_geometries;
        sc->info.bvh2_nodes = sc->has2 ? (uint32_t)sc->bvh2.nodes.size() : 0;
        sc->info.bvh8_nodes = (uint32_t)b8.nodes.size();
        float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        for (uint64_t i = 0; i < 3ull * num_triangles; ++i) {
            const float* p = positions + 3ull * indices[i];
            for (int k = 0; k < 3; ++k) {
                mn[k] = p[k] < mn[k] ? p[k] : mn[k];
                mx[k] = p[k] > mx[k] ? p[k] : mx[k];
            }
        }
        if (num_triangles == 0)
            for (int k = 0; k < 3; ++k) mn[k] = mx[k] = 0.0f;
        for (int k = 0; k < 3; ++k) {
            sc->info.bounds_min[k] = mn[k];
            sc->info.bounds_max[k] = mx[k];
        }
    } catch (const std::bad_alloc&) {
        wfpt_scene_destroy(sc);
        return WFPT_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& ex) {
        wfpt_scene_destroy(sc);
        g_last_error = ex.what();
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    sc->info.build_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    *scene = sc;
    return WFPT_OK;
}

void wfpt_scene_destroy(wfpt_scene* scene) {
    if (!scene) return;
    for (void* b : scene->bufs)
        if (b) cudaFree(b);
    delete scene;
}

wfpt_status wfpt_scene_get_info(const wfpt_scene* scene, wfpt_scene_info* info) {
    WFPT_REQUIRE(scene && info, "null pointer");
    *info = scene->info;
    return WFPT_OK;
}

// Exports of a device-built scene: copies of its device buffers.
static wfpt_status export_device(const void* dnodes, size_t nb, const void* dtris, size_t tb, void* nodes,
                                 size_t* node_bytes, void* triangles, size_t* triangle_bytes) {
    cudaError_t e = cudaSuccess;
    if (nodes) {
        WFPT_REQUIRE(*node_bytes >= nb, "node buffer too small");
        if (nb) e = cudaMemcpy(nodes, dnodes, nb, cudaMemcpyDeviceToHost);
    }
    if (triangles && e == cudaSuccess) {
        WFPT_REQUIRE(*triangle_bytes >= tb, "triangle buffer too small");
        if (tb) e = cudaMemcpy(triangles, dtris, tb, cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) return from_cuda(e);
    *node_bytes = nb;
    *triangle_bytes = tb;
    return WFPT_OK;
}

wfpt_status wfpt_scene_export_bvh2(const wfpt_scene* scene, void* nodes, size_t* node_bytes, void* triangles,
                                   size_t* triangle_bytes) {
    WFPT_REQUIRE(scene && node_bytes && triangle_bytes, "null pointer");
    if (scene->device_built)
        return export_device(scene->bufs[0], scene->dev_bvh2_count * sizeof(wfpt::Bvh2Node), scene->bufs[1],
                             scene->has2 ? scene->dev_ntris * sizeof(wfpt::TriRec) : 0, nodes, node_bytes,
                             triangles, triangle_bytes);
    size_t nb = scene->bvh2.nodes.size() * sizeof(wfpt::Bvh2Node);
    size_t tb = scene->bvh2.tris.size() * sizeof(wfpt::TriRec);
    if (nodes) {
        WFPT_REQUIRE(*node_bytes >= nb, "node buffer too small");
        std::memcpy(nodes, scene->bvh2.nodes.data(), nb);
    }
    if (triangles) {
        WFPT_REQUIRE(*triangle_bytes >= tb, "triangle buffer too small");
        std::memcpy(triangles, scene->bvh2.tris.data(), tb);
    }
    *node_bytes = nb;
    *triangle_bytes = tb;
    return WFPT_OK;
}

wfpt_status wfpt_scene_export_bvh8(const wfpt_scene* scene, void* nodes, size_t* node_bytes, void* triangles,
                                   size_t* triangle_bytes) {
    WFPT_REQUIRE(scene && node_bytes && triangle_bytes, "null pointer");
    if (scene->device_built)
        return export_device(scene->bufs[2], scene->dev_bvh8_count * sizeof(wfpt::Bvh8Node), scene->bufs[3],
                             scene->has8 ? scene->dev_ntris * sizeof(wfpt::TriRec) : 0, nodes, node_bytes,
                             triangles, triangle_bytes);
    size_t nb = scene->bvh8.nodes.size() * sizeof(wfpt::Bvh8Node);
    size_t tb = scene->bvh8.tris.size() * sizeof(wfpt::TriRec);
    if (nodes) {
        WFPT_REQUIRE(*node_bytes >= nb, "node buffer too small");
        std::memcpy(nodes, scene->bvh8.nodes.data(), nb);
    }
    if (triangles) {
        WFPT_REQUIRE(*triangle_bytes >= tb, "triangle buffer too small");
        std::memcpy(triangles, scene->bvh8.tris.data(), tb);
    }
    *node_bytes = nb;
    *triangle_bytes = tb;
    return WFPT_OK;
}

wfpt_status wfpt_trace(const wfpt_scene* scene, int bvh_kind, const wfpt_ray* rays, wfpt_hit* results,
                       const uint32_t* ray_index, uint32_t n, const uint32_t* n_dev, int closest_hit,
                       void* stream) {
    WFPT_REQUIRE(scene, "null scene");
    WFPT_REQUIRE(!scene->host_only, "scene was built host-only and cannot be traced");
    WFPT_REQUIRE(bvh_kind == WFPT_BVH2_FP32 || bvh_kind == WFPT_BVH8_Q8, "unknown bvh kind");
    if (!wfpt::scene_has(scene, bvh_kind)) {
        g_last_error = "scene was built without this BVH kind";
        return WFPT_ERR_UNSUPPORTED;
    }
    WFPT_REQUIRE(n <= kMaxN, "n too large");
    WFPT_REQUIRE(n == 0 || (rays && results), "null buffer");
    return from_cuda(wfpt::launch_trace(scene->dev, bvh_kind, rays, results, ray_index, n, n_dev, closest_hit,
                                        S(stream)));
}

wfpt_status wfpt_trace_sort(const wfpt_scene* scene, int bvh_kind, const wfpt_ray* rays, wfpt_hit* results,
                            uint32_t n, const uint32_t* n_dev, const float scene_min[3], const float scene_max[3],
                            int morton_kind, int reorder, wfpt_ray* rays_out, const int32_t* slot_to_index,
                            int32_t* slot_to_index_out, int32_t* index_to_slot_out, void* keys, uint32_t* indices,
                            int closest_hit, void* scratch, size_t scratch_bytes, void* stream) {
    WFPT_REQUIRE(scene_min && scene_max, "null scene box");
    WFPT_REQUIRE(morton_kind >= WFPT_MORTON_AILA32 && morton_kind <= WFPT_MORTON_6D64, "unknown morton kind");
    WFPT_REQUIRE(!reorder || n == 0 || (rays_out && slot_to_index && slot_to_index_out && index_to_slot_out),
                 "reorder needs the output rays and slot maps");
    const int key_bits = morton_kind == WFPT_MORTON_AILA32 ? 32 : (morton_kind == WFPT_MORTON_6D48 ? 48 : 63);
    const float size[3] = {scene_max[0] - scene_min[0], scene_max[1] - scene_min[1], scene_max[2] - scene_min[2]};
    wfpt_status st = wfpt_morton(rays, n, n_dev, scene_min, size, morton_kind, keys, indices, stream);
    if (st != WFPT_OK) return st;
    if ((st = wfpt_sort_pairs(keys, indices, n, n_dev, key_bits, scratch, scratch_bytes, stream)) != WFPT_OK)
        return st;
    if (reorder) {
        if ((st = wfpt_reorder(indices, rays, rays_out, slot_to_index, slot_to_index_out, index_to_slot_out, n, n_dev,
                               stream)) != WFPT_OK)
            return st;
        return wfpt_trace(scene, bvh_kind, rays_out, results, nullptr, n, n_dev, closest_hit, stream);
    }
    return wfpt_trace(scene, bvh_kind, rays, results, indices, n, n_dev, closest_hit, stream);
}

wfpt_status wfpt_generate_scene(int kind, uint64_t seed, uint32_t num_triangles, float* positions, float* normals,
                                uint32_t* num_vertices, uint32_t* indices, uint32_t* num_triangles_out) {
    WFPT_REQUIRE(num_vertices && num_triangles_out, "null count pointer");
    WFPT_REQUIRE(kind >= 0 && kind <= 3, "unknown scene kind");
    WFPT_REQUIRE(kind != 0 || (num_triangles > 0 && num_triangles < (1u << 27)), "bad triangle count");
    std::vector<float> pos, nrm;
    std::vector<uint32_t> idx;
    try {
        if (!wfpt::generate_scene(kind, seed, num_triangles, pos, nrm, idx)) return invalid("scene generation failed");
    } catch (const std::bad_alloc&) {
        return WFPT_ERR_OUT_OF_MEMORY;
    }
    uint32_t nv = (uint32_t)(pos.size() / 3), nt = (uint32_t)(idx.size() / 3);
    if (positions || normals || indices) {
        WFPT_REQUIRE(*num_vertices >= nv && *num_triangles_out >= nt, "output buffers too small");
        if (positions) std::memcpy(positions, pos.data(), pos.size() * sizeof(float));
        if (normals) std::memcpy(normals, nrm.data(), nrm.size() * sizeof(float));
        if (indices) std::memcpy(indices, idx.data(), idx.size() * sizeof(uint32_t));
    }
    *num_vertices = nv;
    *num_triangles_out = nt;
    return WFPT_OK;
}

}  // extern "C"
