/* C++ facade of libwfpt with the reference's class and method names, so
 * that code written against the reference's Tracer / RayGen / RayBuffer /
 * Renderer switches by changing its includes.  Header-only; every method
 * forwards to one wfpt_* entry point of wfpt.h.
 *
 * As in the reference, the stage methods are synchronous and return the
 * stage's device time in milliseconds (Tracer.cpp:185-225,
 * RayGen.cpp:21-186 wait on a fence and read a GPU timer); errors throw
 * wfpt_cxx::Error instead of asserting.  Buffers are CUDA device memory
 * owned by RayBuffer / RayGen (the reference's vks::Buffer members).
 *
 * Interfaces mirrored: RayBuffer (Ray/RayBuffer.h:22-70), Tracer
 * (Tracer/Tracer.h:60-77), RayGen (Ray/RayGen.h:95-116), Renderer
 * (Renderer/Renderer.h, Renderer.cpp:552-714). */
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "wfpt.h"

namespace wfpt_cxx {

class Error : public std::runtime_error {
public:
    Error(wfpt_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    wfpt_status status;
};

inline void check(wfpt_status s) {
    if (s != WFPT_OK)
        throw Error(s, std::string(wfpt_status_string(s)) + ": " + wfpt_last_error_message());
}

inline void check_cuda(cudaError_t e) {
    if (e != cudaSuccess) throw Error(WFPT_ERR_CUDA, cudaGetErrorString(e));
}

/* Owned device allocation; resize() discards the contents when it grows
 * (as resizeDiscardBuffer, Utils/BufferUtils.cpp:36-42). */
template <typename T>
class DeviceArray {
public:
    DeviceArray() = default;
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    ~DeviceArray() { release(); }
    void resize(size_t n) {
        if (n <= cap_) return;
        release();
        if (n) check_cuda(cudaMalloc(&p_, n * sizeof(T)));
        cap_ = n;
    }
    void release() {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        cap_ = 0;
    }
    T* get() const { return p_; }
    size_t capacity() const { return cap_; }

private:
    T* p_ = nullptr;
    size_t cap_ = 0;
};

/* Times a sequence of stream-ordered calls with CUDA events and waits for
 * it, returning milliseconds. */
class StageTimer {
public:
    explicit StageTimer(cudaStream_t s) : s_(s) {
        check_cuda(cudaEventCreate(&a_));
        check_cuda(cudaEventCreate(&b_));
        check_cuda(cudaEventRecord(a_, s_));
    }
    ~StageTimer() {
        cudaEventDestroy(a_);
        cudaEventDestroy(b_);
    }
    float stop() {
        check_cuda(cudaEventRecord(b_, s_));
        check_cuda(cudaEventSynchronize(b_));
        float ms = 0.0f;
        check_cuda(cudaEventElapsedTime(&ms, a_, b_));
        return ms;
    }

private:
    cudaStream_t s_;
    cudaEvent_t a_ = nullptr, b_ = nullptr;
};

/* RayBuffer: double-buffered rays and slot maps, one result buffer, Morton
 * keys (room for 64-bit keys), sort indices and the sort's storage (the
 * reference's "spine"). */
class RayBuffer {
public:
    RayBuffer() = default;

    void swap() { swap_ = !swap_; }
    int getSize() const { return size_; }
    int getCapacity() const { return capacity_; }
    /* Sets the size; grows (discarding contents) when it exceeds capacity. */
    void resize(int n) {
        if (n > capacity_) {
            rays_[0].resize((size_t)n);
            results_.resize((size_t)n);
            i2s_[0].resize((size_t)n);
            s2i_[0].resize((size_t)n);
            capacity_ = n;
            if (reordering_) resizeReorderingBuffers(true);
        }
        size_ = n;
    }
    void resizeReorderingBuffers(bool reorderRays) {
        reordering_ = reorderRays;
        const size_t n = (size_t)capacity_;
        keys_.resize(n);
        indices_.resize(n);
        spine_.resize(wfpt_sort_scratch_bytes((uint32_t)n, 64));
        if (reorderRays) {
            rays_[1].resize(n);
            i2s_[1].resize(n);
            s2i_[1].resize(n);
        }
    }
    bool getClosestHit() const { return closest_hit_; }
    void setClosestHit(bool closestHit) { closest_hit_ = closestHit; }
    float getRayLength() const { return ray_length_; }
    void setRayLength(float rayLength) { ray_length_ = rayLength; }

    wfpt_ray* getRayBuffer() const { return rays_[swap_ ? 1 : 0].get(); }
    wfpt_ray* getOutRayBuffer() const { return rays_[swap_ ? 0 : 1].get(); }
    wfpt_hit* getResultBuffer() const { return results_.get(); }
    uint32_t* getIndexBuffer() const { return indices_.get(); }
    void* getMortonCodeBuffer() const { return keys_.get(); }
    void* getSpineBuffer() const { return spine_.get(); }
    size_t getSpineBytes() const { return spine_.capacity(); }
    int32_t* getIndexToSlotBuffer() const { return i2s_[swap_ ? 1 : 0].get(); }
    int32_t* getOutIndexToSlotBuffer() const { return i2s_[swap_ ? 0 : 1].get(); }
    int32_t* getSlotToIndexBuffer() const { return s2i_[swap_ ? 1 : 0].get(); }
    int32_t* getOutSlotToIndexBuffer() const { return s2i_[swap_ ? 0 : 1].get(); }

private:
    int capacity_ = 0, size_ = 0;
    DeviceArray<wfpt_ray> rays_[2];
    DeviceArray<wfpt_hit> results_;
    DeviceArray<int32_t> i2s_[2], s2i_[2];
    DeviceArray<uint64_t> keys_;
    DeviceArray<uint32_t> indices_;
    DeviceArray<unsigned char> spine_;
    bool closest_hit_ = true, reordering_ = false, swap_ = false;
    float ray_length_ = 0.0f;
};

/* Scene (the reference's acceleration structure): owns a wfpt_scene. */
class Scene {
public:
    Scene(const float* positions, uint32_t num_vertices, const uint32_t* indices, uint32_t num_triangles,
          const uint32_t* geometry_first_triangle = nullptr, uint32_t num_geometries = 0,
          int bvh_kinds_mask = (1 << WFPT_BVH2_FP32) | (1 << WFPT_BVH8_Q8)) {
        check(wfpt_scene_create(positions, num_vertices, indices, num_triangles, geometry_first_triangle,
                                num_geometries, bvh_kinds_mask, &s_));
    }
    /* Geometry already in device memory: both BVHs built on the GPU
     * (wfpt_scene_create_device). */
    static Scene fromDevice(const float* positions_dev, uint32_t num_vertices, const uint32_t* indices_dev,
                            uint32_t num_triangles, const uint32_t* geometry_first_triangle = nullptr,
                            uint32_t num_geometries = 0,
                            int bvh_kinds_mask = (1 << WFPT_BVH2_FP32) | (1 << WFPT_BVH8_Q8),
                            cudaStream_t stream = nullptr) {
        wfpt_scene* s = nullptr;
        check(wfpt_scene_create_device(positions_dev, num_vertices, indices_dev, num_triangles,
                                       geometry_first_triangle, num_geometries, bvh_kinds_mask, stream, &s));
        return Scene(s);
    }
    Scene(Scene&& o) noexcept : s_(o.s_) { o.s_ = nullptr; }
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;
    ~Scene() {
        if (s_) wfpt_scene_destroy(s_);
    }
    const wfpt_scene* get() const { return s_; }
    wfpt_scene_info info() const {
        wfpt_scene_info i;
        check(wfpt_scene_get_info(s_, &i));
        return i;
    }

private:
    explicit Scene(wfpt_scene* s) : s_(s) {}
    wfpt_scene* s_ = nullptr;
};

/* Tracer: trace / traceSort over a RayBuffer. */
class Tracer {
public:
    void init(cudaStream_t stream = nullptr) { stream_ = stream; }
    void setAccelerationStructure(const Scene& scene, int bvh_kind = WFPT_BVH8_Q8) {
        scene_ = scene.get();
        kind_ = bvh_kind;
    }
    /* The reference's spelling of the same method (Tracer.h:70). */
    void setAccererationStructure(const Scene& scene, int bvh_kind = WFPT_BVH8_Q8) {
        setAccelerationStructure(scene, bvh_kind);
    }
    void setMortonKind(int morton_kind) { morton_ = morton_kind; }

    float trace(RayBuffer& rays) {
        StageTimer t(stream_);
        check(wfpt_trace(scene_, kind_, rays.getRayBuffer(), rays.getResultBuffer(), nullptr,
                         (uint32_t)rays.getSize(), nullptr, rays.getClosestHit() ? 1 : 0, stream_));
        return t.stop();
    }

    float traceSort(RayBuffer& rays, const float sceneMinPos[3], const float sceneMaxPos[3], bool reorderRays) {
        std::array<float, 4> times;
        return traceSort(rays, sceneMinPos, sceneMaxPos, reorderRays, times);
    }

    /* times: Morton codes, radix sort, reorder (0 without), trace. */
    float traceSort(RayBuffer& rays, const float sceneMinPos[3], const float sceneMaxPos[3], bool reorderRays,
                    std::array<float, 4>& times) {
        const uint32_t n = (uint32_t)rays.getSize();
        rays.resizeReorderingBuffers(reorderRays);
        const float size[3] = {sceneMaxPos[0] - sceneMinPos[0], sceneMaxPos[1] - sceneMinPos[1],
                               sceneMaxPos[2] - sceneMinPos[2]};
        const int bits = morton_ == WFPT_MORTON_AILA32 ? 32 : (morton_ == WFPT_MORTON_6D48 ? 48 : 63);
        {
            StageTimer t(stream_);
            check(wfpt_morton(rays.getRayBuffer(), n, nullptr, sceneMinPos, size, morton_,
                              rays.getMortonCodeBuffer(), rays.getIndexBuffer(), stream_));
            times[0] = t.stop();
        }
        {
            StageTimer t(stream_);
            check(wfpt_sort_pairs(rays.getMortonCodeBuffer(), rays.getIndexBuffer(), n, nullptr, bits,
                                  rays.getSpineBuffer(), rays.getSpineBytes(), stream_));
            times[1] = t.stop();
        }
        times[2] = 0.0f;
        if (reorderRays) {
            StageTimer t(stream_);
            check(wfpt_reorder(rays.getIndexBuffer(), rays.getRayBuffer(), rays.getOutRayBuffer(),
                               rays.getSlotToIndexBuffer(), rays.getOutSlotToIndexBuffer(),
                               rays.getOutIndexToSlotBuffer(), n, nullptr, stream_));
            times[2] = t.stop();
            rays.swap();
        }
        {
            StageTimer t(stream_);
            check(wfpt_trace(scene_, kind_, rays.getRayBuffer(), rays.getResultBuffer(),
                             reorderRays ? nullptr : rays.getIndexBuffer(), n, nullptr,
                             rays.getClosestHit() ? 1 : 0, stream_));
            times[3] = t.stop();
        }
        return times[0] + times[1] + times[2] + times[3];
    }

private:
    cudaStream_t stream_ = nullptr;
    const wfpt_scene* scene_ = nullptr;
    int kind_ = WFPT_BVH8_Q8;
    int morton_ = WFPT_MORTON_AILA32;
};

/* RayGen: seeds, primary / shadow / path ray generation.  Owns the seeds,
 * the pixel table of the current extent and the path-ray counter. */
class RayGen {
public:
    void init(cudaStream_t stream = nullptr) { stream_ = stream; }

    float initSeeds(int numberOfPixels, int frameIndex = 1) {
        seeds_.resize((size_t)numberOfPixels);
        StageTimer t(stream_);
        check(wfpt_init_seeds(seeds_.get(), (uint32_t)numberOfPixels, frameIndex, stream_));
        return t.stop();
    }

    /* RayGen::primary: one ray per pixel in pixel-table order. */
    float primary(RayBuffer& orays, const wfpt_camera& camera, int width, int height, int sampleIndex) {
        set_extent(width, height);
        float m[16];
        check(wfpt_camera_screen_to_world(camera.position, camera.rotation_deg, camera.fov_deg,
                                          (float)width / (float)height, camera.znear, camera.zfar, m));
        orays.resize(width * height);
        StageTimer t(stream_);
        check(wfpt_raygen_primary(m, i2p_.get(), orays.getRayBuffer(), camera.position, sampleIndex, width, height,
                                  camera.zfar, stream_));
        check_cuda(cudaMemcpyAsync(orays.getSlotToIndexBuffer(), i2p_.get(), (size_t)width * height * 4,
                                   cudaMemcpyDeviceToDevice, stream_));
        return t.stop();
    }

    /* RayGen::shadow: numberOfSamples rays per input ray of the batch
     * [batchBegin, batchEnd); seeds are indexed batch-locally. */
    float shadow(RayBuffer& orays, RayBuffer& irays, int batchBegin, int batchEnd, int numberOfSamples,
                 const float light[3], float lightRadius) {
        const int bs = batchEnd - batchBegin;
        orays.resize(bs * numberOfSamples);
        orays.setClosestHit(false);
        StageTimer t(stream_);
        check(wfpt_raygen_shadow(seeds_.get(), irays.getRayBuffer(), irays.getResultBuffer(), orays.getRayBuffer(),
                                 orays.getSlotToIndexBuffer(), orays.getIndexToSlotBuffer(), light, lightRadius,
                                 batchBegin, bs, nullptr, numberOfSamples, stream_));
        return t.stop();
    }

    /* RayGen::path: compacted bounce rays; reads the count back and sets
     * orays' size, as the reference does (RayGen.cpp:178-183). */
    float path(RayBuffer& orays, RayBuffer& irays, float* decreases, const wfpt_geometry* geometries,
               float albedo = 0.8f) {
        const uint32_t n = (uint32_t)irays.getSize();
        orays.resize((int)n);
        orays.setClosestHit(true);
        count_.resize(1);
        scratch_.resize(wfpt_raygen_path_scratch_bytes(n));
        StageTimer t(stream_);
        check(wfpt_raygen_path(seeds_.get(), geometries, irays.getRayBuffer(), orays.getRayBuffer(),
                               irays.getSlotToIndexBuffer(), orays.getSlotToIndexBuffer(), irays.getResultBuffer(),
                               decreases, count_.get(), n, nullptr, russian_roulette_ ? 1 : 0, albedo,
                               scratch_.get(), scratch_.capacity(), stream_));
        const float ms = t.stop();
        uint32_t c = 0;
        check_cuda(cudaMemcpy(&c, count_.get(), 4, cudaMemcpyDeviceToHost));
        orays.resize((int)c);
        return ms;
    }

    bool getRussianRoulette() const { return russian_roulette_; }
    void setRussianRoulette(bool russianRoulette) { russian_roulette_ = russianRoulette; }
    uint32_t* seedPtr() const { return seeds_.get(); }
    const int32_t* indexToPixelPtr() const { return i2p_.get(); }

private:
    void set_extent(int w, int h) {
        if (w == w_ && h == h_) return;
        std::vector<int32_t> a((size_t)w * h), b((size_t)w * h);
        check(wfpt_pixel_table(w, h, a.data(), b.data()));
        i2p_.resize(a.size());
        check_cuda(cudaMemcpy(i2p_.get(), a.data(), a.size() * 4, cudaMemcpyHostToDevice));
        w_ = w;
        h_ = h;
    }
    cudaStream_t stream_ = nullptr;
    DeviceArray<uint32_t> seeds_, count_;
    DeviceArray<int32_t> i2p_;
    DeviceArray<unsigned char> scratch_;
    bool russian_roulette_ = false;
    int w_ = 0, h_ = 0;
};

/* Renderer: the whole frame (Renderer::render) and its performance
 * figures (Renderer::get*Performance, Renderer.cpp:660-714: Mrays/s =
 * rays * 1e-3 / ms). */
class Renderer {
public:
    explicit Renderer(const wfpt_renderer_config* config = nullptr) { check(wfpt_renderer_create(config, &r_)); }
    Renderer(const Renderer&) = delete;
    Renderer& operator=(const Renderer&) = delete;
    ~Renderer() { wfpt_renderer_destroy(r_); }

    void setConfig(const wfpt_renderer_config& c) { check(wfpt_renderer_set_config(r_, &c)); }
    void setScene(const Scene& scene, const wfpt_geometry* geometries, const float light[3],
                  const float background[3], const float* scene_min = nullptr, const float* scene_max = nullptr) {
        check(wfpt_renderer_set_scene(r_, scene.get(), geometries, scene_min, scene_max, light, background));
    }
    void resetFrameIndex() { wfpt_renderer_reset_frame_index(r_); }
    void render(const wfpt_camera& camera, int width, int height, float* pixels, float* framePixels,
                cudaStream_t stream = nullptr) {
        check(wfpt_renderer_render(r_, &camera, width, height, pixels, framePixels, stream));
    }
    wfpt_render_stats stats() {
        wfpt_render_stats s;
        check(wfpt_renderer_get_stats(r_, &s));
        return s;
    }
    /* Renderer::getNumberOf*Rays (Renderer.cpp:660-674) of the last frame. */
    unsigned long long getNumberOfPrimaryRays() { return stats().num_primary_rays; }
    unsigned long long getNumberOfShadowRays() { return stats().num_shadow_rays; }
    unsigned long long getNumberOfPathRays() { return stats().num_path_rays; }
    unsigned long long getNumberOfRays() {
        const wfpt_render_stats s = stats();
        return s.num_primary_rays + s.num_shadow_rays + s.num_path_rays;
    }
    /* Renderer::get*TraceTime (Renderer.cpp:676-690), in ms: filled when the
     * config's timing option is on (the reference's benchmark mode), else 0. */
    float getPrimaryTraceTime() { return stats().primary_trace_ms; }
    float getShadowTraceTime() { return stats().shadow_trace_ms; }
    float getPathTraceTime() { return stats().path_trace_ms; }
    float getTraceTime() {
        const wfpt_render_stats s = stats();
        return s.primary_trace_ms + s.shadow_trace_ms + s.path_trace_ms;
    }
    /* Renderer::get*TracePerformance (Renderer.cpp:692-706): Mrays/s = rays *
     * 1e-3 / trace ms, 0 when the trace time is 0 (timing off). */
    float getPrimaryTracePerformance() { return perf(stats().num_primary_rays, getPrimaryTraceTime()); }
    float getShadowTracePerformance() { return perf(stats().num_shadow_rays, getShadowTraceTime()); }
    float getPathTracePerformance() { return perf(stats().num_path_rays, getPathTraceTime()); }
    float getTracePerformance() { return perf(getNumberOfRays(), getTraceTime()); }
    /* Mrays/s of the last frame over all rays against the whole frame's
     * device time (no counterpart: the reference divides by trace time). */
    float getFramePerformance() {
        const wfpt_render_stats s = stats();
        return perf(s.num_primary_rays + s.num_shadow_rays + s.num_path_rays, s.frame_ms);
    }
    /* Renderer::getShadowSortLogs / getPathSortLogs (Renderer.cpp:708-714). */
    wfpt_sort_log getShadowSortLog(int depth) { return stats().shadow_sort_logs[depth]; }
    wfpt_sort_log getPathSortLog(int depth) { return stats().path_sort_logs[depth]; }
    wfpt_renderer* get() const { return r_; }

private:
    static float perf(unsigned long long rays, float ms) { return ms == 0.0f ? 0.0f : (float)(rays * 1.0e-3 / ms); }
    wfpt_renderer* r_ = nullptr;
};

}  // namespace wfpt_cxx
