/*
 * wfpt.h — C ABI of the GB300 wavefront path tracer (libwfpt.so).
 *
 * This header is the drop-in boundary for the wavefront stage chain of
 * JJH1101/VulkanWaveFrontPathTracer: ray generation -> Morton keys -> LSD
 * key/value radix sort -> ray reorder -> BVH traversal -> shading,
 * reconstruction and accumulation.  Each stage entry point replaces one
 * reference compute shader plus the host method that dispatches it; the
 * reference passes raw 64-bit buffer device addresses in push-constant
 * structs, and this ABI passes the same buffers as plain device pointers.
 *
 * Conventions (all entry points):
 *  - every pointer named *_dev or typed as a record array is CUDA device
 *    memory owned by the caller unless stated otherwise;
 *  - calls are stream-ordered and asynchronous on `stream` (a cudaStream_t,
 *    NULL = legacy default stream) and return a wfpt_status for argument
 *    and launch errors; device-side errors (a bounded wait that gave up)
 *    are latched in a device status word read by wfpt_device_status();
 *  - `n` is the element count known on the host; where an entry point also
 *    takes `const uint32_t* n_dev`, a non-NULL n_dev makes the kernel read
 *    the count from device memory (clamped to `n`, which is then the
 *    capacity).  This is what lets a whole frame run without host readbacks
 *    and be captured in one CUDA graph.
 *  - no entry point allocates device memory except the scene and renderer
 *    constructors; scratch is passed in by the caller.
 */
#ifndef WFPT_H_
#define WFPT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WFPT_ABI_VERSION 1

/* ------------------------------------------------------------------ types */

/* Ray record, 32 bytes.  Same field order as `struct Ray`
 * (projects/WaveFrontPathTracer/Ray/Ray.h:32-37, ray.glsl:9-14). */
typedef struct wfpt_ray {
    float origin[3];
    float tmin;
    float direction[3];
    float tmax;
} wfpt_ray;

/* Hit record, 16 bytes.  Same field order as `struct RayResult`
 * (Ray/Ray.h:39-44, ray.glsl:16-21).  Miss = {-1, -1, -1.0f, 0}
 * (trace.comp:77-82); packed_bary = packUnorm2x16(u, v) where the hit point
 * is (1-u-v)*v0 + u*v1 + v*v2 (trace.comp:74). */
typedef struct wfpt_hit {
    int32_t primitive_id;
    int32_t geometry_id;
    float t;
    uint32_t packed_bary;
} wfpt_hit;

/* Per-geometry shading table entry, 16 bytes: `struct Geometry`
 * (geometrytypes.glsl:9-12).  vertex_addr points at vkglTF::Vertex records
 * (96 bytes = 6 float4: pos.xyz normal.x | normal.yz uv.xy | ...,
 * base/VulkanglTFModel.h:221-228); index_addr at uint32 triangle indices
 * already offset by the primitive's firstIndex. */
typedef struct wfpt_geometry {
    uint64_t vertex_addr;
    uint64_t index_addr;
} wfpt_geometry;

typedef enum wfpt_status {
    WFPT_OK = 0,
    WFPT_ERR_INVALID_ARGUMENT = 1,
    WFPT_ERR_CUDA = 2,
    WFPT_ERR_OUT_OF_MEMORY = 3,
    WFPT_ERR_TIMEOUT = 4,       /* a bounded device-side wait gave up */
    WFPT_ERR_UNSUPPORTED = 5,
    WFPT_ERR_SCRATCH_TOO_SMALL = 6,
    WFPT_ERR_DEVICE_BOUNDS = 7  /* a device-side bounds check fired */
} wfpt_status;

/* Acceleration structure flavours. */
typedef enum wfpt_bvh_kind {
    WFPT_BVH2_FP32 = 0, /* plain form: binary BVH, FP32 child boxes (64-B nodes) */
    WFPT_BVH8_Q8 = 1    /* chosen form: 8-wide BVH, 8-bit quantised child boxes (80-B nodes) */
} wfpt_bvh_kind;

/* Morton key layouts.  AILA32 is the reference's only method
 * (computeMortonCodesAila32.comp:38-88; 32-bit keys).  The 6-D forms are
 * additions: origin and normalised direction interleaved per bit level,
 * 48 bits (8 bits per axis) or 63 bits (origin 11 bits per axis, direction
 * 10 bits per axis) in 64-bit keys. */
typedef enum wfpt_morton_kind {
    WFPT_MORTON_AILA32 = 0,
    WFPT_MORTON_6D48 = 1,
    WFPT_MORTON_6D64 = 2
} wfpt_morton_kind;

/* Ray types of the renderer (Renderer.h:72-77). */
typedef enum wfpt_ray_type {
    WFPT_PRIMARY_RAYS = 0,
    WFPT_SHADOW_RAYS = 1,
    WFPT_PATH_RAYS = 2
} wfpt_ray_type;

/* --------------------------------------------------------------- library */

int wfpt_abi_version(void);
const char* wfpt_status_string(wfpt_status status);
/* Message of the last CUDA error seen by this library on this thread. */
const char* wfpt_last_error_message(void);
/* Synchronises the current device, returns and clears the device status
 * word: bit 0 = a bounded wait timed out (WFPT_ERR_TIMEOUT), bit 1 = a
 * bounds check fired.  *flags may be NULL. */
wfpt_status wfpt_device_status(uint32_t* flags);
/* Number of kernels this library has launched since it was loaded (for
 * benchmarks; no counterpart in the reference). */
uint64_t wfpt_kernel_launch_count(void);

/* Process-wide tuning knobs (no counterpart in the reference; set by the
 * autotuner).  Keys:
 *   "trace.bvh8.refill"    refill a persistent warp when this many lanes
 *                          are idle (1..32, default 8)
 *   "trace.bvh8.postpone"  per-lane triangle tests (coop 0): postpone a
 *                          node's triangle tests while fewer than this many
 *                          lanes have triangles (0..32, 0 = off)
 *   "trace.bvh8.coop"      1 = the warp tests all of its lanes' pending
 *                          triangles together, 32 at a time (default);
 *                          0 = each lane tests its own.  Closest hits are
 *                          identical; an any-hit ray may report a different
 *                          (equally valid) occluder
 *   "trace.bvh8.batch"     cooperative tests of closest-hit rays: run them
 *                          once this many are pending across the warp's
 *                          node steps (1..32, default 24; 1 = after every
 *                          loop iteration)
 *   "trace.bvh8.steps"     cooperative tests of closest-hit rays: node steps
 *                          a lane takes per loop iteration while its steps
 *                          hand it no triangles (1..8, default 2)
 *   "trace.bvh8.any_batch" the same for any-hit rays (default 1)
 *   "trace.bvh8.any_steps" the same for any-hit rays (default 3)
 *   "sort.tiles"           radix sort tile size: 0 = by problem size
 *                          (default), 1 = small tiles, 2 = large tiles,
 *                          3 = extra-large tiles (32-bit keys; 64-bit keys
 *                          take the large ones)
 *   "sort.digit_bits"      radix digit width per pass: 8 (default) or 4
 *   "build.bvh8.collapse"  BVH8 collapse of scenes built afterwards: 1 = SAH
 *                          dynamic programme (default), 0 = greedy fill
 *   "build.ploc.radius"    device build: clusters on either side searched
 *                          for a nearest neighbour (1..64, default 8)
 *   "build.bvh8.tri_cost"  triangle-test cost relative to a node step in the
 *                          SAH collapse, percent (1..10000, default 20)
 *   "debug.fail_alloc_after"  fault injection: n >= 0 makes the renderer's
 *                          device allocation after n more successful ones
 *                          report WFPT_ERR_OUT_OF_MEMORY (nothing is
 *                          allocated); -1 (default) off
 *   "debug.alloc_count"   read only (wfpt_tune_get): device and pinned host
 *                          allocations the library has made in this process
 *   "trace.count"         1 = launch the counting traversal kernels, which
 *                          accumulate the counters read by wfpt_trace_counters
 *   "renderer.shadow_slots"  shadow batches a renderer runs at once in an
 *                          overlapped shadow pass: 0 (default) = planned
 *                          from free device memory, 1..8 = that many
 *                          (capped by the batches a pass can need)
 * Unknown keys and out-of-range values return WFPT_ERR_INVALID_ARGUMENT. */
wfpt_status wfpt_tune_set(const char* key, int64_t value);
wfpt_status wfpt_tune_get(const char* key, int64_t* value);
/* Self-test of the device-side failure detection (no reference counterpart;
 * the reference waits on fences and asserts).  Runs one bounded device wait
 * that cannot succeed -- which = 0: a radix sort pass whose decoupled
 * look-back waits on a tile that nothing publishes; 1: the path-ray
 * compaction's look-back likewise -- and returns what wfpt_device_status
 * then reports: WFPT_ERR_TIMEOUT when the wait gave up as designed (the
 * status word is cleared and the context stays usable).  Synchronises the
 * device; takes one to a few seconds. */
wfpt_status wfpt_selftest_wait_timeout(int which);

/* Counters of the counting traversal kernels (synchronises): out[0] node
 * visits, out[1] triangle tests, out[2] rays, out[3] persistent-warp loop
 * iterations; reset != 0 zeroes them. */
wfpt_status wfpt_trace_counters(uint64_t out[4], int reset);

/* ------------------------------------------------------ host-side helpers */

/* PixelTable::recalculate (Ray/PixelTable.cpp:21-99): index<->pixel bijection
 * (8x8 blocks in Morton order, pixels swizzled inside each block, remainder
 * stripes appended).  Host buffers of width*height int32 each. */
wfpt_status wfpt_pixel_table(int width, int height, int32_t* index_to_pixel,
                             int32_t* pixel_to_index);

/* inverse(P * V) for the reference's first-person camera
 * (RayGen.cpp:93; base/camera.hpp:23-45 view, :108-120 perspective with
 * depth 0..1 and P[1][1] *= -1).  Column-major 4x4 like glm::mat4. */
wfpt_status wfpt_camera_screen_to_world(const float position[3],
                                        const float rotation_deg[3],
                                        float fov_deg, float aspect,
                                        float znear, float zfar,
                                        float screen_to_world[16]);

/* --------------------------------------------------------- stage kernels */

/* initSeeds.comp:7-40 + RayGen::initSeeds (RayGen.cpp:21-44):
 * seeds[i] = tea(i, frame_index, 16). */
wfpt_status wfpt_init_seeds(uint32_t* seeds, uint32_t n, int frame_index,
                            void* stream);

/* raygenPrimary.comp:44-85 + RayGen::primary (RayGen.cpp:80-105).
 * rays[i] for pixel index_to_pixel[i]; jitter = Halton(2,3) of
 * sample_index, identical for every pixel. */
wfpt_status wfpt_raygen_primary(const float screen_to_world[16],
                                const int32_t* index_to_pixel, wfpt_ray* rays,
                                const float origin[3], int sample_index,
                                int width, int height, float max_dist,
                                void* stream);

/* computeMortonCodesAila32.comp:24-95 + Tracer::computeMortonCodes
 * (Tracer.cpp:22-37).  keys is uint32_t[n] for AILA32, uint64_t[n] for the
 * 6-D kinds; indices[i] = i. */
wfpt_status wfpt_morton(const wfpt_ray* rays, uint32_t n, const uint32_t* n_dev,
                        const float scene_min[3], const float scene_size[3],
                        int morton_kind, void* keys, uint32_t* indices,
                        void* stream);

/* Scratch needed by wfpt_sort_pairs for up to max_n pairs
 * (replaces vrdxGetSorterKeyValueStorageRequirements,
 * external/vulkan_radix_sort/vk_radix_sort.h:2547-2562). */
size_t wfpt_sort_scratch_bytes(uint32_t max_n, int key_bits);

/* Stable LSD key/value radix sort with 8-bit digits
 * (replaces Tracer::radixSort, Tracer.cpp:39-78, and vrdxCmdSortKeyValue,
 * vk_radix_sort.h:2579-2585).  Keys are uint32_t when key_bits <= 32, else
 * uint64_t; only the low key_bits bits are sorted on (ceil(key_bits/8)
 * passes).  The result is left in keys/values, like the reference.  Values
 * are uint32.  Ordering equals a stable sort by key.  The call enqueues a
 * memset of the scratch, a histogram kernel and one kernel per pass; the
 * pass kernels are launched with programmatic stream serialisation after
 * the library's own previous kernel (they start as it drains and wait for
 * it before reading), so a stream capture records programmatic edges
 * between them.  Work the caller enqueues after the sort starts only when
 * the sort has completed, as with any stream-ordered call. */
wfpt_status wfpt_sort_pairs(void* keys, uint32_t* values, uint32_t n,
                            const uint32_t* n_dev, int key_bits, void* scratch,
                            size_t scratch_bytes, void* stream);

/* reorderRays.comp:27-46 + Tracer::reorderRays (Tracer.cpp:80-98):
 * out_rays[i] = in_rays[idx[i]]; out_slot_to_index[i] =
 * in_slot_to_index[idx[i]]; out_index_to_slot[out_slot_to_index[i]] = i.
 * ray_index must be a permutation of [0, n); out_index_to_slot must have
 * room for every value in in_slot_to_index (pixel indices in a renderer,
 * which can exceed n in a compacted wavefront). */
wfpt_status wfpt_reorder(const uint32_t* ray_index, const wfpt_ray* in_rays,
                         wfpt_ray* out_rays, const int32_t* in_slot_to_index,
                         int32_t* out_slot_to_index, int32_t* out_index_to_slot,
                         uint32_t n, const uint32_t* n_dev, void* stream);

/* The reorder gather for records other than the 32-byte wfpt_ray (ray
 * records carrying a payload; 48 B is the wide layout the sort/reorder
 * microbenchmark uses).  No reference counterpart: reorderRays.comp:37-45
 * moves 32-byte Ray records only.  out_records[i] = in_records[ray_index[i]]
 * for records of record_bytes = 16, 32, 48 or 64 bytes; both record buffers
 * 16-byte aligned.  The slot maps follow wfpt_reorder when given; pass all
 * three as NULL for a plain gather. */
wfpt_status wfpt_reorder_records(const uint32_t* ray_index, const void* in_records,
                                 void* out_records, uint32_t record_bytes,
                                 const int32_t* in_slot_to_index,
                                 int32_t* out_slot_to_index, int32_t* out_index_to_slot,
                                 uint32_t n, const uint32_t* n_dev, void* stream);

/* raygenShadow.comp:68-137 + RayGen::shadow (RayGen.cpp:107-133).  Seeds
 * are indexed by batch-local task index like the reference. */
wfpt_status wfpt_raygen_shadow(const uint32_t* seeds, const wfpt_ray* in_rays,
                               const wfpt_hit* in_results, wfpt_ray* out_rays,
                               int32_t* out_slot_to_index,
                               int32_t* out_index_to_slot, const float light[3],
                               float light_radius, int batch_begin,
                               int batch_size, const uint32_t* n_in_dev,
                               int num_samples, void* stream);

/* Scratch for wfpt_raygen_path's ordered compaction. */
size_t wfpt_raygen_path_scratch_bytes(uint32_t max_n);

/* raygenPath.comp:78-169 + RayGen::path (RayGen.cpp:135-186).  Cosine
 * bounce for every hit; the compaction keeps input order (the reference's
 * subgroup-ballot + atomicAdd order is nondeterministic) and *out_count_dev
 * receives the number of output rays (written, not accumulated).  albedo is
 * the reference's hard-coded 0.8 (raygenPath.comp:138) made a parameter. */
wfpt_status wfpt_raygen_path(uint32_t* seeds, const wfpt_geometry* geometries,
                             const wfpt_ray* in_rays, wfpt_ray* out_rays,
                             const int32_t* in_index_to_pixel,
                             int32_t* out_index_to_pixel,
                             const wfpt_hit* in_results, float* decreases,
                             uint32_t* out_count_dev, uint32_t n,
                             const uint32_t* n_dev, int russian_roulette,
                             float albedo, void* scratch, size_t scratch_bytes,
                             void* stream);

/* Largest n accepted by wfpt_raygen_path_static. */
#define WFPT_RAYGEN_PATH_STATIC_MAX_RAYS 16777216u

/* wfpt_raygen_path without caller scratch; no counterpart in the reference
 * (the reference's raygenPath.comp appends through an atomic counter and
 * needs no scratch).
 *
 * For callers that cannot hand the library device memory: an engine whose
 * device memory is all owned by its own allocator (for example a Vulkan
 * renderer that exports a fixed set of buffers to CUDA and has none spare),
 * or code on a latency-critical path where cudaMalloc / cudaFree would
 * synchronise the device.  This call allocates nothing: its compaction
 * scratch is a fixed 256 KiB array in the library's device image
 * (one per device), enough for n <= WFPT_RAYGEN_PATH_STATIC_MAX_RAYS.
 *
 * - Results equal wfpt_raygen_path's for the same inputs.
 * - n above WFPT_RAYGEN_PATH_STATIC_MAX_RAYS is rejected with
 *   WFPT_ERR_INVALID_ARGUMENT before anything is launched; use
 *   wfpt_raygen_path with caller scratch for larger wavefronts.
 * - The tile ticket and the per-tile look-back states must start at zero;
 *   the call clears them itself, stream-ordered on `stream`, before its
 *   kernel.  The caller clears nothing.  *out_count_dev is written, not
 *   accumulated.
 * - The first call in each CUDA context (each device's primary context,
 *   and again after cudaDeviceReset) looks up the array's device address
 *   with cudaGetSymbolAddress; make that first call outside any stream
 *   capture.  A first call made while `stream` is capturing launches
 *   nothing and returns WFPT_ERR_INVALID_ARGUMENT with a message saying so.
 *   The address is cached per context (by its unique id), so a later
 *   context on the same device never uses a stale address.
 * - All calls on one device share the one array: calls that overlap in time
 *   (two streams with no event ordering them, or two host threads) race on
 *   it and give wrong output or WFPT_ERR_TIMEOUT from wfpt_device_status.
 *   Issue them on one stream or order them with events. */
wfpt_status wfpt_raygen_path_static(uint32_t* seeds, const wfpt_geometry* geometries,
                                    const wfpt_ray* in_rays, wfpt_ray* out_rays,
                                    const int32_t* in_index_to_pixel,
                                    int32_t* out_index_to_pixel,
                                    const wfpt_hit* in_results, float* decreases,
                                    uint32_t* out_count_dev, uint32_t n,
                                    const uint32_t* n_dev, int russian_roulette,
                                    float albedo, void* stream);

/* reconstructSmooth.comp:34-96 + Renderer::reconstructSmooth
 * (Renderer.cpp:201-223).  pixels/decreases are float4 per pixel. */
wfpt_status wfpt_reconstruct_smooth(const wfpt_ray* rays, const wfpt_hit* results,
                                    const int32_t* index_to_pixel, float* pixels,
                                    const float* decreases,
                                    const wfpt_geometry* geometries,
                                    const float light[3],
                                    const float background[3], uint32_t n,
                                    const uint32_t* n_dev, int num_samples,
                                    void* stream);

/* reconstructShadow.comp:30-61 + Renderer::reconstructShadow
 * (Renderer.cpp:225-245).  n_in_dev (nullable) clamps the batch to the
 * device-side count of input rays. */
wfpt_status wfpt_reconstruct_shadow(const wfpt_hit* shadow_results,
                                    const int32_t* index_to_pixel,
                                    const int32_t* index_to_slot,
                                    const float* in_pixels, float* out_pixels,
                                    int batch_begin, int batch_size,
                                    const uint32_t* n_in_dev, int num_samples,
                                    int replace, void* stream);

/* countRayHits.comp:24-50 + Renderer::computeRayHits (Renderer.cpp:54-91):
 * *count_dev += number of results with primitive_id >= 0 (caller zeroes). */
wfpt_status wfpt_count_hits(const wfpt_hit* results, uint32_t n,
                            const uint32_t* n_dev, uint32_t* count_dev,
                            void* stream);

/* interpolateColors.comp:71-98 + Renderer::interpolateColors
 * (Renderer.cpp:106-122): running mean over frames + Reinhard tone map. */
wfpt_status wfpt_interpolate_colors(float* frame_pixels, float* pixels,
                                    uint32_t num_pixels, int frame_index,
                                    float key_value, float white_point,
                                    void* stream);

/* interpolateColors.comp:71-98 with the running mean kept in double
 * (FP64 per-pixel accumulation over frames): accum holds one double4
 * per pixel (xyz the mean, w unused; 32-byte aligned), written on every
 * frame (frame 1: the frame's colour), blended on later frames with
 * a = 1/frame, b = a * (frame - 1) in double; pixels receives the mean
 * rounded to float (w as the float path writes it) and frame_pixels its
 * Reinhard tone map. */
wfpt_status wfpt_interpolate_colors_fp64(float* frame_pixels, float* pixels,
                                         double* accum, uint32_t num_pixels,
                                         int frame_index, float key_value,
                                         float white_point, void* stream);

/* vks::util::clearBuffer / clearBufferTimed with a 32-bit pattern
 * (Utils/BufferUtils.cpp; used by Renderer::initDecreases with 1.0f). */
wfpt_status wfpt_fill_u32(void* dst, uint32_t pattern, size_t count_u32,
                          void* stream);

/* ----------------------------------------------------------------- scene */

typedef struct wfpt_scene wfpt_scene;

typedef struct wfpt_scene_info {
    uint32_t num_triangles;
    uint32_t num_geometries;
    uint32_t bvh2_nodes;
    uint32_t bvh8_nodes;
    float bounds_min[3];
    float bounds_max[3];
    double build_ms;
} wfpt_scene_info;

/* Builds the acceleration structures on the host and uploads them; replaces
 * the driver BLAS/TLAS build (WaveFrontPathTracer.cpp:202-457).
 * positions: host float[3*num_vertices]; indices: host uint32[3*num_triangles];
 * geometry_first_triangle: host uint32[num_geometries] (ascending, first = 0)
 * or NULL for one geometry.  primitive_id in hits is the triangle index
 * within its geometry, geometry_id the geometry index (trace.comp:71-72).
 * bvh_kinds_mask: bit (1<<WFPT_BVH2_FP32) and/or (1<<WFPT_BVH8_Q8), plus
 * WFPT_SCENE_HOST_ONLY to build on the host without uploading (such a scene
 * can be exported but not traced). */
#define WFPT_SCENE_HOST_ONLY 0x100
/* bvh_kinds_mask flag: upload the mesh and build both BVHs on the device
 * (wfpt_scene_create_device) instead of on the host.  Scenes of fewer than
 * two triangles are built on the host either way. */
#define WFPT_SCENE_DEVICE_BUILD 0x200
wfpt_status wfpt_scene_create(const float* positions, uint32_t num_vertices,
                              const uint32_t* indices, uint32_t num_triangles,
                              const uint32_t* geometry_first_triangle,
                              uint32_t num_geometries, int bvh_kinds_mask,
                              wfpt_scene** scene);
/* Device build from geometry already in device memory: positions_dev
 * float[3*num_vertices], indices_dev uint32[3*num_triangles];
 * geometry_first_triangle stays a host array.  No reference counterpart
 * beyond the AS build it replaces (WaveFrontPathTracer.cpp:202-457, driver
 * BLAS build with PREFER_FAST_TRACE): the BVH2 by PLOC clustering of
 * Morton-sorted triangle centroids, the BVH8 by the same SAH collapse as the
 * host build (knobs "build.bvh8.*").  Hits equal those of a host-built scene
 * of the same mesh (the traversal result does not depend on the tree).
 * Runs on `stream` and returns when the scene is ready; out-of-range
 * triangle indices return WFPT_ERR_INVALID_ARGUMENT.  Exports of such a
 * scene copy its device buffers. */
wfpt_status wfpt_scene_create_device(const float* positions_dev, uint32_t num_vertices,
                                     const uint32_t* indices_dev, uint32_t num_triangles,
                                     const uint32_t* geometry_first_triangle,
                                     uint32_t num_geometries, int bvh_kinds_mask,
                                     void* stream, wfpt_scene** scene);
void wfpt_scene_destroy(wfpt_scene* scene);
wfpt_status wfpt_scene_get_info(const wfpt_scene* scene, wfpt_scene_info* info);
/* Host copies of the BVH2 (FP32 nodes, 64 B each) and its triangle table
 * (48 B each), for host-side checks.  Pass NULL buffers to get sizes. */
wfpt_status wfpt_scene_export_bvh2(const wfpt_scene* scene, void* nodes,
                                   size_t* node_bytes, void* triangles,
                                   size_t* triangle_bytes);
/* Host copies of the BVH8 (80-B compressed nodes) and its triangle table. */
wfpt_status wfpt_scene_export_bvh8(const wfpt_scene* scene, void* nodes,
                                   size_t* node_bytes, void* triangles,
                                   size_t* triangle_bytes);

/* trace.comp:27-86 + Tracer::trace (Tracer.cpp:185-207) with a software
 * stack traversal instead of rayQuery.  closest_hit = 0 terminates on the
 * first hit (gl_RayFlagsTerminateOnFirstHitEXT).  ray_index (nullable) is
 * the indirect index: thread i traces ray ray_index[i] and writes
 * results[ray_index[i]].  A ray with tmax < tmin misses. */
wfpt_status wfpt_trace(const wfpt_scene* scene, int bvh_kind, const wfpt_ray* rays,
                       wfpt_hit* results, const uint32_t* ray_index, uint32_t n,
                       const uint32_t* n_dev, int closest_hit, void* stream);

/* Tracer::traceSort (Tracer.cpp:214-225) as one stream-ordered call:
 * Morton keys of the rays over the box [scene_min, scene_max] (wfpt_morton
 * with morton_kind), stable key sort of (key, index) (wfpt_sort_pairs with
 * 32, 48 or 63 key bits), then
 *  - reorder != 0: wfpt_reorder into rays_out / slot_to_index_out /
 *    index_to_slot_out and trace those (the reordered buffers become the
 *    wavefront, as RayBuffer::swap does); results follow the reordered
 *    slots;
 *  - reorder == 0: trace the rays in sorted order through the indirect
 *    index; results land at each ray's own slot (rays_out and the out maps
 *    may be null).
 * keys: n u32 (WFPT_MORTON_AILA32) or n u64 (6-D kinds); indices: n u32;
 * scratch: at least wfpt_sort_scratch_bytes(n, 64) bytes. */
wfpt_status wfpt_trace_sort(const wfpt_scene* scene, int bvh_kind, const wfpt_ray* rays,
                            wfpt_hit* results, uint32_t n, const uint32_t* n_dev,
                            const float scene_min[3], const float scene_max[3],
                            int morton_kind, int reorder, wfpt_ray* rays_out,
                            const int32_t* slot_to_index, int32_t* slot_to_index_out,
                            int32_t* index_to_slot_out, void* keys, uint32_t* indices,
                            int closest_hit, void* scratch, size_t scratch_bytes,
                            void* stream);

/* ------------------------------------------------------ synthetic scenes */

/* Seeded scene generators standing in for the reference's glTF scenes.
 *  kind 0: triangle soup in the unit cube (num_triangles given),
 *  kind 1: courtyard (box room, 48 cylinders, clutter, ~262K triangles),
 *  kind 2: city block (64x64 boxes, subdivided displaced faces, ~3M),
 *  kind 3: city block scaled to about num_triangles.
 * Output is an indexed mesh with per-vertex normals; call twice, first
 * with NULL buffers to get the counts. */
wfpt_status wfpt_generate_scene(int kind, uint64_t seed, uint32_t num_triangles,
                                float* positions, float* normals,
                                uint32_t* num_vertices, uint32_t* indices,
                                uint32_t* num_triangles_out);

/* -------------------------------------------------------------- renderer */

typedef struct wfpt_renderer wfpt_renderer;

/* Renderer options; keys and defaults follow the reference's env options
 * (Environment/AppEnvironment.cpp:10-43, Renderer.cpp:300-308) plus the
 * additions morton_kind, bvh_kind, albedo, use_graph, path_sort_skip,
 * shadow_overlap, primary_bvh_kind. */
typedef struct wfpt_renderer_config {
    int ray_type;                   /* Renderer.rayType */
    int num_primary_samples;        /* Renderer.numberOfPrimarySamples, 1..1024 */
    int num_shadow_samples;         /* Renderer.numberOfShadowSamples, 1..1024 */
    float shadow_radius;            /* Renderer.shadowRadius, (0,100] */
    int recursion_depth;            /* Renderer.recursionDepth, 0..8 */
    float key_value;                /* Renderer.keyValue, (0,2] */
    float white_point;              /* Renderer.whitePoint, (0,2] */
    int russian_roulette;           /* Renderer.russianRoulette (no effect, as in the reference) */
    int sort_shadow_rays;           /* Renderer.sortShadowRays */
    int reorder_shadow_rays;        /* Renderer.reorderShadowRays */
    int sort_path_rays;             /* Renderer.sortPathRays */
    int reorder_path_rays;          /* Renderer.reorderPathRays */
    int morton_kind;                /* Renderer.mortonMethod: wfpt_morton_kind */
    int bvh_kind;                   /* wfpt_bvh_kind used by trace */
    float albedo;                   /* path albedo, reference hard-codes 0.8 */
    int use_graph;                  /* capture the frame in a CUDA graph */
    int path_sort_skip;             /* bit b set: bounce b+1 traces its path rays
                                       unsorted even when sort_path_rays is on
                                       (per-bounce reordering; 0..255, default 0) */
    int shadow_overlap;             /* 1 (default): each pass's shadow rays are
                                       traced and reconstructed on a second
                                       stream while the next bounce's path rays
                                       are generated, sorted and traced; 0: one
                                       stream in the reference's order.  Results
                                       are identical. */
    int primary_bvh_kind;           /* BVH traversed by the primary pass (camera
                                       rays and their shadow rays): -1 (default)
                                       = bvh_kind, else a wfpt_bvh_kind.  On
                                       coherent camera rays the FP32 BVH2 is the
                                       faster one (the autotuner's choice). */
    int timing;                     /* Application.mode "benchmark" with
                                       Benchmark.printSortLogs: 0 (default) off;
                                       1: the frame's stages are launched
                                       directly on one stream (use_graph and
                                       shadow_overlap are not applied) with CUDA
                                       event pairs around them, which fill the
                                       per-type trace times and the sort logs of
                                       wfpt_render_stats; a sorted pass also
                                       traces its rays unsorted first to log the
                                       unsorted trace time, as the reference
                                       does (Renderer.cpp:255-297).  Pixels and
                                       ray counts are the same as without. */
    int accumulate_fp64;            /* 0 (default): the running mean over frames
                                       in float, as interpolateColors.comp; 1:
                                       the mean kept in a double-precision
                                       buffer of the renderer (32 bytes per
                                       pixel), `pixels` gets its rounding to
                                       float and the tone map reads that. */
} wfpt_renderer_config;

void wfpt_renderer_config_default(wfpt_renderer_config* config);

typedef struct wfpt_camera {
    float position[3];
    float rotation_deg[3];
    float fov_deg;
    float znear;
    float zfar;
} wfpt_camera;

/* SortLog (Renderer.h:29-46): one pass's ray count and the device times of
 * its Morton keys, sort, reorder, sorted trace (traceSort's trace) and
 * unsorted trace, in milliseconds, summed over the frame's primary samples. */
typedef struct wfpt_sort_log {
    uint64_t ray_count;
    float morton_ms;
    float sort_ms;
    float reorder_ms;
    float trace_sort_ms;
    float trace_ms;
} wfpt_sort_log;

/* Statistics of the last frame (Renderer.cpp:660-714, Renderer.h:29-46). */
typedef struct wfpt_render_stats {
    uint64_t num_primary_rays;
    uint64_t num_shadow_rays;
    uint64_t num_path_rays;
    uint32_t path_rays_per_bounce[8];
    uint32_t shadow_hits_per_pass[9];
    float frame_ms;                 /* device time of the whole frame */
    /* With config.timing = 1 (else 0): getPrimaryTraceTime (raygenPrimary +
     * trace), getShadowTraceTime (raygenShadow + trace or traceSort, every
     * batch), getPathTraceTime (raygenPath + trace or traceSort), in ms;
     * RT PERF of a ray type = its ray count * 1e-3 / its trace time. */
    int timed;
    float primary_trace_ms;
    float shadow_trace_ms;
    float path_trace_ms;
    /* shadowSortLogs[0..depth] (0: the primary pass's shadow rays, b + 1:
     * bounce b's) and pathSortLogs[0..depth-1]; times are filled for sorted
     * passes, ray counts for every pass. */
    wfpt_sort_log shadow_sort_logs[9];
    wfpt_sort_log path_sort_logs[8];
    /* Shadow batches of the last frame that ran at once: the renderer's
     * memory planner gives overlapped shadow passes up to
     * min(batches, 8) slots, as many as fit in half of the free device
     * memory (knob renderer.shadow_slots forces a count); 1 when the
     * batches ran one after another. */
    int shadow_batch_slots;
} wfpt_render_stats;

wfpt_status wfpt_renderer_create(const wfpt_renderer_config* config,
                                 wfpt_renderer** renderer);
void wfpt_renderer_destroy(wfpt_renderer* renderer);
wfpt_status wfpt_renderer_set_config(wfpt_renderer* renderer,
                                     const wfpt_renderer_config* config);
/* Renderer::setScene (Renderer.cpp:523-550).  geometries is a device array
 * of num_geometries wfpt_geometry entries owned by the caller. */
wfpt_status wfpt_renderer_set_scene(wfpt_renderer* renderer, const wfpt_scene* scene,
                                    const wfpt_geometry* geometries,
                                    const float scene_min[3],
                                    const float scene_max[3], const float light[3],
                                    const float background[3]);
void wfpt_renderer_reset_frame_index(wfpt_renderer* renderer);
/* Renderer::render (Renderer.cpp:552-654).  pixels and frame_pixels are
 * device float4[width*height] owned by the caller; frame_pixels receives the
 * tone-mapped frame, pixels the running mean. */
wfpt_status wfpt_renderer_render(wfpt_renderer* renderer, const wfpt_camera* camera,
                                 int width, int height, float* pixels,
                                 float* frame_pixels, void* stream);
/* Ray counts are read back from the device, so this synchronises. */
wfpt_status wfpt_renderer_get_stats(wfpt_renderer* renderer, wfpt_render_stats* stats);

/* ---- batched render requests (no counterpart in the reference, which
 * renders one view per Renderer::render call) ---------------------------
 * Many requests -- different scenes, resolutions, sample counts and depths
 * -- rendered as one captured CUDA graph: every request's frame is recorded
 * once, spread over `streams` graph branches so that small requests run
 * side by side, and each wfpt_batch_render call replays it with every
 * request's camera and frame index read from device memory.  A request's
 * output equals what a wfpt_renderer with the same config, scene and camera
 * renders, frame for frame. */
typedef struct wfpt_request {
    const wfpt_scene* scene;
    const wfpt_geometry* geometries; /* device geometry table of the scene */
    float light[3];
    float background[3];
    wfpt_camera camera;
    int width, height;
    wfpt_renderer_config config;     /* use_graph is ignored */
    float* pixels;                   /* device, width*height float4: accumulated image */
    float* frame_pixels;             /* device, width*height float4: this frame */
} wfpt_request;

typedef struct wfpt_batch wfpt_batch;

/* Allocates every request's buffers and records the batch graph (not
 * inside a stream capture).  streams: graph branches, 1..16. */
wfpt_status wfpt_batch_create(const wfpt_request* requests, uint32_t count, int streams,
                              wfpt_batch** batch);
void wfpt_batch_destroy(wfpt_batch* batch);
/* One frame of every request, stream-ordered on `stream`.  cameras
 * (nullable, `count` entries) replaces the requests' cameras for this and
 * later calls. */
wfpt_status wfpt_batch_render(wfpt_batch* batch, const wfpt_camera* cameras, void* stream);
/* Request i's ray counts of the last batch frame (synchronises);
 * frame_ms is the device time of the whole batch. */
wfpt_status wfpt_batch_get_stats(wfpt_batch* batch, uint32_t i, wfpt_render_stats* stats);
/* Kernel launches one wfpt_batch_render makes (the graph's kernel nodes). */
uint64_t wfpt_batch_kernels(const wfpt_batch* batch);
void wfpt_batch_reset_frame_index(wfpt_batch* batch);

#ifdef __cplusplus
}
#endif

#endif /* WFPT_H_ */
