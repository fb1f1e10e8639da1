// Entry points of oracle/_ref/libref.so: the reference's own shader and host
// code, compiled by oracle/ref_build.py, behind plain C functions that the
// tests call to pin the restatement in oracle.cpp (test infrastructure only).
// Each entry fills the shader's push constants as the reference's host code
// does (Ray/RayGen.cpp, Tracer/Tracer.cpp, Renderer/Renderer.cpp) and
// dispatches ceil(n / local size) workgroups.  Buffers are host arrays whose
// addresses stand in for the buffer device addresses.
#include <cstdint>
#include <cstring>
#include <vector>

#include "camera.hpp"
#include "glsl_shim.hpp"

namespace ref_initSeeds {
using namespace glsl;
#include "gen/initSeeds.inc"
}
namespace ref_raygenPrimary {
using namespace glsl;
#include "gen/raygenPrimary.inc"
}
namespace ref_mortonAila32 {
using namespace glsl;
#include "gen/mortonAila32.inc"
}
namespace ref_reorderRays {
using namespace glsl;
#include "gen/reorderRays.inc"
}
namespace ref_raygenShadow {
using namespace glsl;
#include "gen/raygenShadow.inc"
}
namespace ref_raygenPath {
using namespace glsl;
#include "gen/raygenPath.inc"
}
namespace ref_reconstructSmooth {
using namespace glsl;
#include "gen/reconstructSmooth.inc"
}
namespace ref_reconstructShadow {
using namespace glsl;
#include "gen/reconstructShadow.inc"
}
namespace ref_countRayHits {
using namespace glsl;
#include "gen/countRayHits.inc"
}
namespace ref_interpolateColors {
using namespace glsl;
#include "gen/interpolateColors.inc"
}

static uint64_t A(const void* p) { return (uint64_t)(uintptr_t)p; }

template <class NS_PC>
static void zero(NS_PC& pc) {
    std::memset(static_cast<void*>(&pc), 0, sizeof(pc));
}

#define DISPATCH(NS, n) glsl::dispatch(glsl::groups_for((n), NS::kLocalSizeX), NS::kLocalSizeX, NS::shader_main, NS::kUsesFibers)

extern "C" {

// RayGen::initSeeds (RayGen.cpp:21-44).
void ref_init_seeds(uint32_t* seeds, int n, int frame_index) {
    namespace R = ref_initSeeds;
    zero(R::pc);
    R::pc.seedAddr = A(seeds);
    R::pc.numberOfPixels = n;
    R::pc.frameIndex = frame_index;
    DISPATCH(R, (uint64_t)n);
}

// RayGen::primary (RayGen.cpp:80-105); m is screenToWorld, column-major.
void ref_raygen_primary(const float m[16], const int32_t* index_to_pixel, float* rays, const float origin[3],
                        int sample_index, int w, int h, float max_dist) {
    namespace R = ref_raygenPrimary;
    zero(R::pc);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) R::pc.screenToWorld[c][r] = m[c * 4 + r];
    R::pc.indexToPixelAddr = A(index_to_pixel);
    R::pc.rayBufferAddr = A(rays);
    R::pc.origin = glsl::vec3(origin[0], origin[1], origin[2]);
    R::pc.sampleIndex = sample_index;
    R::pc.size = glsl::ivec2(w, h);
    R::pc.maxDist = max_dist;
    DISPATCH(R, (uint64_t)w * h);
}

// Tracer::computeMortonCodes (Tracer.cpp:22-37).
void ref_morton_aila32(const float* rays, uint32_t n, const float smin[3], const float ssize[3], uint32_t* keys,
                       uint32_t* indices) {
    namespace R = ref_mortonAila32;
    zero(R::pc);
    R::pc.rayAddr = A(rays);
    R::pc.mortonCodeAddr = A(keys);
    R::pc.rayIndexAddr = A(indices);
    R::pc.numberOfRays = n;
    R::pc.sceneMin = glsl::vec3(smin[0], smin[1], smin[2]);
    R::pc.sceneSize = glsl::vec3(ssize[0], ssize[1], ssize[2]);
    DISPATCH(R, n);
}

// Tracer::reorderRays (Tracer.cpp:80-98).
void ref_reorder(const uint32_t* ray_index, const float* in_rays, float* out_rays, const int32_t* in_s2i,
                 int32_t* out_s2i, int32_t* out_i2s, int n) {
    namespace R = ref_reorderRays;
    zero(R::pc);
    R::pc.rayIndexAddr = A(ray_index);
    R::pc.inRayAddr = A(in_rays);
    R::pc.outRayAddr = A(out_rays);
    R::pc.inSlotToIndexAddr = A(in_s2i);
    R::pc.outSlotToIndexAddr = A(out_s2i);
    R::pc.outIndexToSlotAddr = A(out_i2s);
    R::pc.numberOfRays = n;
    DISPATCH(R, (uint64_t)n);
}

// RayGen::shadow (RayGen.cpp:107-133): batch_size input rays from
// batch_begin, S output rays each.
void ref_raygen_shadow(const uint32_t* seeds, const float* in_rays, const int32_t* in_results, float* out_rays,
                       int32_t* out_s2i, int32_t* out_i2s, const float light[3], float radius, int batch_begin,
                       int batch_size, int S) {
    namespace R = ref_raygenShadow;
    zero(R::pc);
    R::pc.seedAddr = A(seeds);
    R::pc.inputRayAddr = A(in_rays);
    R::pc.outputRayAddr = A(out_rays);
    R::pc.inputResultAddr = A(in_results);
    R::pc.outputSlotToIndexAddr = A(out_s2i);
    R::pc.outputIndexToSlotAddr = A(out_i2s);
    R::pc.light = glsl::vec3(light[0], light[1], light[2]);
    R::pc.lightRadius = radius;
    R::pc.batchBegin = batch_begin;
    R::pc.batchSize = batch_size;
    R::pc.numberOfSamples = S;
    DISPATCH(R, (uint64_t)batch_size);
}

// RayGen::path (RayGen.cpp:135-186); geometries is the Geometry table
// {vertexAddr, indexAddr}; *count must hold 0 on entry.  Returns *count.
uint32_t ref_raygen_path(uint32_t* seeds, const uint64_t* geometries, const float* in_rays, float* out_rays,
                         const int32_t* in_i2p, int32_t* out_i2p, const int32_t* in_results, float* decreases,
                         uint32_t* count, int n) {
    namespace R = ref_raygenPath;
    zero(R::pc);
    R::pc.seedAddr = A(seeds);
    R::pc.geometryAddr = A(geometries);
    R::pc.inputRayAddr = A(in_rays);
    R::pc.outputRayAddr = A(out_rays);
    R::pc.inputIndexToPixelAddr = A(in_i2p);
    R::pc.outputIndexToPixelAddr = A(out_i2p);
    R::pc.inputResultAddr = A(in_results);
    R::pc.decreaseAddr = A(decreases);
    R::pc.numberOfOutputRayAddr = A(count);
    R::pc.numberOfInputRays = n;
    R::pc.russianRoulette = 0;
    DISPATCH(R, (uint64_t)n);
    return *count;
}

// Renderer::reconstructSmooth (Renderer.cpp:201-223).
void ref_reconstruct_smooth(const float* rays, const int32_t* results, const int32_t* i2p, float* pixels,
                            const float* decreases, const uint64_t* geometries, const float light[3],
                            const float background[3], int n, int spp) {
    namespace R = ref_reconstructSmooth;
    zero(R::pc);
    R::pc.rayAddr = A(rays);
    R::pc.resultAddr = A(results);
    R::pc.idxToPixelAddr = A(i2p);
    R::pc.pixelAddr = A(pixels);
    R::pc.decreaseAddr = A(decreases);
    R::pc.geometryAddr = A(geometries);
    R::pc.light = glsl::vec3(light[0], light[1], light[2]);
    R::pc.numberOfRays = n;
    R::pc.backgroundColor = glsl::vec3(background[0], background[1], background[2]);
    R::pc.numberOfSamples = spp;
    DISPATCH(R, (uint64_t)n);
}

// Renderer::reconstructShadow (Renderer.cpp:225-245).
void ref_reconstruct_shadow(const int32_t* shadow_results, const int32_t* i2p, const int32_t* i2s,
                            const float* in_pixels, float* out_pixels, int batch_begin, int batch_size, int S,
                            int replace) {
    namespace R = ref_reconstructShadow;
    zero(R::pc);
    R::pc.outputResultAddr = A(shadow_results);
    R::pc.indexToPixelAddr = A(i2p);
    R::pc.indexToSlotAddr = A(i2s);
    R::pc.inPixelAddr = A(in_pixels);
    R::pc.outPixelAddr = A(out_pixels);
    R::pc.batchBegin = batch_begin;
    R::pc.batchSize = batch_size;
    R::pc.numberOfSamples = S;
    R::pc.replace = replace;
    DISPATCH(R, (uint64_t)batch_size);
}

// Renderer::computeRayHits (Renderer.cpp:54-91): the counter starts at 0.
uint32_t ref_count_hits(const int32_t* results, int n) {
    namespace R = ref_countRayHits;
    uint32_t hits = 0;
    zero(R::pc);
    R::pc.rayResultAddr = A(results);
    R::pc.rayHitAddr = A(&hits);
    R::pc.numberOfRays = n;
    DISPATCH(R, (uint64_t)n);
    return hits;
}

// Renderer::interpolateColors (Renderer.cpp:106-122).
void ref_interpolate_colors(float* frame_pixels, float* pixels, int n, int frame_index, float key, float white) {
    namespace R = ref_interpolateColors;
    zero(R::pc);
    R::pc.framePixelAddr = A(frame_pixels);
    R::pc.pixelAddr = A(pixels);
    R::pc.numberOfPixels = n;
    R::pc.frameIndex = frame_index;
    R::pc.keyValue = key;
    R::pc.whitePoint = white;
    DISPATCH(R, (uint64_t)n);
}

// PixelTable::recalculate (PixelTable.cpp:21-126): the two lookup tables
// that it uploads, built by the reference's own loops (lines 39-99).
void ref_pixel_table(int w, int h, int32_t* index_to_pixel, int32_t* pixel_to_index) {
    struct {
        int x, y;
    } size = {w, h};
    std::vector<int> idxtopos(size.x * size.y);
    std::vector<int> postoidx(size.x * size.y);
#include "gen/pixel_table_body.inc"
    std::memcpy(index_to_pixel, idxtopos.data(), idxtopos.size() * sizeof(int));
    std::memcpy(pixel_to_index, postoidx.data(), postoidx.size() * sizeof(int));
}

// The camera set-up of WaveFrontPathTracer.cpp:98-101 (first-person camera,
// setPerspective, setPosition, setRotation) and RayGen.cpp:93's
// screenToWorld = inverse(perspective * view), column-major out[c*4 + r].
void ref_camera_screen_to_world(const float pos[3], const float rot[3], float fov, float aspect, float zn, float zf,
                                float out[16], float view[16], float proj[16]) {
    Camera camera;
    camera.type = Camera::CameraType::firstperson;
    camera.setPerspective(fov, aspect, zn, zf);
    camera.setPosition(glm::vec3(pos[0], pos[1], pos[2]));
    camera.setRotation(glm::vec3(rot[0], rot[1], rot[2]));
    glm::mat4 m = glm::inverse(camera.matrices.perspective * camera.matrices.view);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            out[c * 4 + r] = m[c][r];
            if (view) view[c * 4 + r] = camera.matrices.view[c][r];
            if (proj) proj[c * 4 + r] = camera.matrices.perspective[c][r];
        }
}

}  // extern "C"
