// Ray generation, shading, reconstruction and accumulation kernels.
//
// Each kernel restates one reference compute shader
// (shaders/glsl/WaveFrontPathTracer/*.comp) with the reference's buffer
// layouts and per-element semantics.  Launch shape: one thread per work
// item, 256-thread blocks; every kernel honours an optional device-side
// element count so that a frame can run without host readbacks.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <mutex>

#include "common.cuh"
#include "morton.cuh"
#include "stages.cuh"

namespace wfpt {

cudaError_t status_stages(uint32_t* out) { return read_and_clear_status(out); }

static std::atomic<uint64_t> g_launches{0};
void count_launch(uint32_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

static std::atomic<uint64_t> g_allocs{0};
cudaError_t dev_malloc(void** p, size_t bytes) {
    g_allocs.fetch_add(1, std::memory_order_relaxed);
    return cudaMalloc(p, bytes);
}
cudaError_t host_malloc(void** p, size_t bytes) {
    g_allocs.fetch_add(1, std::memory_order_relaxed);
    return cudaMallocHost(p, bytes);
}
uint64_t alloc_count() { return g_allocs.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------- seeds
// initSeeds.comp:7-19 (TEA, 16 rounds) and :31-40.
__device__ __forceinline__ uint32_t tea(uint32_t v0, uint32_t v1, uint32_t rounds) {
    uint32_t s0 = 0u;
    for (uint32_t n = 0; n < rounds; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

// fp (nullable): when given, the frame index comes from the device-side
// frame parameters of a captured frame graph.
__global__ void k_init_seeds(uint32_t* __restrict__ seeds, uint32_t n, uint32_t frame,
                             const FrameParams* __restrict__ fp) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (fp) frame = (uint32_t)fp->frame_index;
    if (i < n) seeds[i] = tea(i, frame, 16);
}

// ------------------------------------------------------------- primary
// raygenPrimary.comp:11-22 (radical inverse in float, same operation order).
__device__ __forceinline__ float halton(int i, int base) {
    float r = 0.0f;
    float f = __fdiv_rn(1.0f, (float)base);
    int j = i;
    while (j > 0) {
        r = __fadd_rn(r, __fmul_rn(f, (float)(j % base)));
        j /= base;
        f = __fdiv_rn(f, (float)base);
    }
    return r;
}

struct Mat4 {
    float m[16];  // column-major, m[c*4 + r]
};

// raygenPrimary.comp:57-84.  fp (nullable): camera, far plane and sample
// index (pass + spp * (frame_index - 1)) come from the device-side frame
// parameters of a captured frame graph instead of the arguments.
__global__ void k_raygen_primary(Mat4 s2w, const int32_t* __restrict__ index_to_pixel,
                                 float4* __restrict__ rays, float ox, float oy, float oz,
                                 int sample_index, int width, int height, float max_dist,
                                 const FrameParams* __restrict__ fp, int pass, int spp) {
    uint32_t task = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t num_pixels = (uint32_t)width * (uint32_t)height;
    if (task >= num_pixels) return;
    if (fp) {
#pragma unroll
        for (int k = 0; k < 16; ++k) s2w.m[k] = fp->s2w[k];
        ox = fp->eye[0];
        oy = fp->eye[1];
        oz = fp->eye[2];
        max_dist = fp->zfar;
        sample_index = pass + spp * (fp->frame_index - 1);
    }
    int pixel = index_to_pixel[task];
    int sx = pixel % width;
    int sy = pixel / width;
    float hx = halton(sample_index, 2);
    float hy = halton(sample_index, 3);
    float x = __fadd_rn((float)sx, hx);
    float y = __fadd_rn((float)sy, hy);
    float v0 = __fsub_rn(__fdiv_rn(__fmul_rn(2.0f, x), (float)width), 1.0f);
    float v1 = __fsub_rn(__fdiv_rn(__fmul_rn(2.0f, y), (float)height), 1.0f);
    float v2 = 0.0f, v3 = 1.0f;
    float w4[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float acc = __fmul_rn(s2w.m[0 * 4 + r], v0);
        acc = __fadd_rn(acc, __fmul_rn(s2w.m[1 * 4 + r], v1));
        acc = __fadd_rn(acc, __fmul_rn(s2w.m[2 * 4 + r], v2));
        acc = __fadd_rn(acc, __fmul_rn(s2w.m[3 * 4 + r], v3));
        w4[r] = acc;
    }
    f3 world = mk(__fdiv_rn(w4[0], w4[3]), __fdiv_rn(w4[1], w4[3]), __fdiv_rn(w4[2], w4[3]));
    f3 o = mk(ox, oy, oz);
    f3 d = normalize(sub(world, o));
    rays[2 * task + 0] = make_float4(ox, oy, oz, 0.0f);
    rays[2 * task + 1] = make_float4(d.x, d.y, d.z, max_dist);
}

// -------------------------------------------------------------- shadow
// raygenShadow.comp:10-20.
__device__ __forceinline__ void jenkins_mix(uint32_t& a, uint32_t& b, uint32_t& c) {
    a -= b; a -= c; a ^= (c >> 13);
    b -= c; b -= a; b ^= (a << 8);
    c -= a; c -= b; c ^= (b >> 13);
    a -= b; a -= c; a ^= (c >> 12);
    b -= c; b -= a; b ^= (a << 16);
    c -= a; c -= b; c ^= (b >> 5);
    a -= b; a -= c; a ^= (c >> 3);
    b -= c; b -= a; b ^= (a << 10);
    c -= a; c -= b; c ^= (b >> 15);
}

// raygenShadow.comp:22-40.
__device__ __forceinline__ void sobol2d(uint32_t i, float& x, float& y) {
    uint32_t r1 = 0, r2 = 0;
    for (uint32_t v1 = 1u << 31, v2 = 3u << 30; i > 0u; i >>= 1) {
        if ((i & 1u) == 1u) {
            r1 ^= v1;
            r2 ^= v2 << 1;
        }
        v1 |= v1 >> 1;
        v2 ^= v2 >> 1;
    }
    x = __fdiv_rn(__uint2float_rn(r1), 4294967296.0f);
    y = __fdiv_rn(__uint2float_rn(r2), 4294967296.0f);
}

// raygenShadow.comp:82-136.  Output rays of input task t occupy
// [S*t, S*t+S) of the batch-local output buffer.
__global__ void k_raygen_shadow(const uint32_t* __restrict__ seeds,
                                const float4* __restrict__ in_rays,
                                const int4* __restrict__ in_results, float4* __restrict__ out_rays,
                                int32_t* __restrict__ out_s2i, int32_t* __restrict__ out_i2s,
                                float lx, float ly, float lz, float radius, int batch_begin,
                                int batch_size, const uint32_t* __restrict__ n_in_dev, int S) {
    uint32_t task = blockIdx.x * blockDim.x + threadIdx.x;
    int size = batch_size;
    if (n_in_dev != nullptr) {
        int avail = (int)*n_in_dev - batch_begin;
        if (avail < size) size = avail;
    }
    if ((int)task >= size) return;
    uint32_t seed = seeds[task];
    float4 r0 = in_rays[2 * (batch_begin + task) + 0];
    float4 r1 = in_rays[2 * (batch_begin + task) + 1];
    int4 res = in_results[batch_begin + task];
    uint32_t ha = seed + task, hb = 0x9e3779b9u, hc = 0x9e3779b9u;
    jenkins_mix(ha, hb, hc);
    jenkins_mix(ha, hb, hc);
    const float two_m32 = 2.3283064365386963e-10f;  // exp2(-32)
    f3 offset = mk(__fmul_rn(__uint2float_rn(ha), two_m32), __fmul_rn(__uint2float_rn(hb), two_m32),
                   __fmul_rn(__uint2float_rn(hc), two_m32));
    int tri = res.x;
    float t = __int_as_float(res.z);
    const float EPS = 1.0e-5f;
    float back = fmaxf(__fsub_rn(t, EPS), 0.0f);
    f3 origin = add(mk(r0.x, r0.y, r0.z), mul(mk(r1.x, r1.y, r1.z), back));
    if (tri == -1) origin = mk(0.0f, 0.0f, 0.0f);
    f3 light = mk(lx, ly, lz);
    int ray_index = S * (int)task;
    for (int i = 0; i < S; ++i) {
        float px, py;
        sobol2d((uint32_t)i, px, py);
        float pz = __fdiv_rn(__fadd_rn((float)i, 0.5f), (float)S);
        px = __fadd_rn(px, offset.x);
        py = __fadd_rn(py, offset.y);
        pz = __fadd_rn(pz, offset.z);
        if (px >= 1.0f) px = __fsub_rn(px, 1.0f);
        if (py >= 1.0f) py = __fsub_rn(py, 1.0f);
        if (pz >= 1.0f) pz = __fsub_rn(pz, 1.0f);
        f3 pos = mk(__fsub_rn(__fmul_rn(2.0f, px), 1.0f), __fsub_rn(__fmul_rn(2.0f, py), 1.0f),
                    __fsub_rn(__fmul_rn(2.0f, pz), 1.0f));
        f3 target = add(light, mul(pos, radius));
        f3 dir = sub(target, origin);
        f3 nd = tri == -1 ? mk(1.0f, 0.0f, 0.0f) : normalize(dir);
        float tmax = tri == -1 ? -1.0f : length(dir);
        out_rays[2 * ray_index + 0] = make_float4(origin.x, origin.y, origin.z, EPS);
        out_rays[2 * ray_index + 1] = make_float4(nd.x, nd.y, nd.z, tmax);
        out_s2i[ray_index] = ray_index;
        out_i2s[ray_index] = ray_index;
        ++ray_index;
    }
}

// ------------------------------------------------------- unpackTriangle
// geometrytypes.glsl:18-47: interpolated, normalised vertex normal from the
// 96-byte vkglTF::Vertex records (normal = (d0.w, d1.x, d1.y)).
__device__ __forceinline__ f3 unpack_normal(const wfpt_geometry* __restrict__ geoms, int geom,
                                            int prim, uint32_t packed_bary) {
    wfpt_geometry g = geoms[geom];
    const uint32_t* __restrict__ idx = reinterpret_cast<const uint32_t*>(g.index_addr);
    const float4* __restrict__ verts = reinterpret_cast<const float4*>(g.vertex_addr);
    float bu, bv;
    unpack_unorm2x16(packed_bary, bu, bv);
    float c0 = __fsub_rn(__fsub_rn(1.0f, bu), bv);
    float cs[3] = {c0, bu, bv};
    f3 n = mk(0.0f, 0.0f, 0.0f);
    uint32_t tri = (uint32_t)prim * 3u;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        uint32_t off = idx[tri + i] * 6u;
        float4 d0 = verts[off + 0];
        float4 d1 = verts[off + 1];
        f3 ni = mul(mk(d0.w, d1.x, d1.y), cs[i]);
        n = (i == 0) ? ni : add(n, ni);
    }
    return normalize(n);
}

// ---------------------------------------------------------------- path
// raygenPath.comp:16-26 (LCG) and :32-49 (Duff et al. ONB, cosine sample).
__device__ __forceinline__ uint32_t lcg(uint32_t& seed) {
    seed = 1103515245u * seed + 12345u;
    return seed & 0x00FFFFFFu;
}
__device__ __forceinline__ float randf(uint32_t& seed) {
    return __fdiv_rn((float)lcg(seed), (float)0x01000000);
}
__device__ __forceinline__ f3 cosine_random_vector(float r0, float r1, f3 n) {
    float sn, cs;
    sincos_2pi(r1, sn, cs);
    float radius = __fsqrt_rn(r0);
    float x = __fmul_rn(radius, sn);
    float z = __fmul_rn(radius, cs);
    float y = __fsqrt_rn(__fsub_rn(1.0f, r0));
    float s = (n.z >= 0.0f) ? 1.0f : -1.0f;
    float a = __fdiv_rn(-1.0f, __fadd_rn(s, n.z));
    float b = __fmul_rn(__fmul_rn(n.x, n.y), a);
    f3 u = mk(__fadd_rn(1.0f, __fmul_rn(__fmul_rn(__fmul_rn(s, n.x), n.x), a)), __fmul_rn(s, b),
              -__fmul_rn(s, n.x));
    f3 v = mk(b, __fadd_rn(s, __fmul_rn(__fmul_rn(n.y, n.y), a)), -n.y);
    return add(add(mul(u, x), mul(v, z)), mul(n, y));
}

// Ordered compaction state: per-tile words (2-bit flag | 30-bit value).
constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;

// Exclusive prefix of `count` over tiles 0..tile-1 by decoupled look-back.
// Called by every thread of the block; returns the prefix in all threads.
// Warp 0 reads 32 predecessors per round trip (lane k: tile - 1 - k), finds
// the nearest one that published its inclusive prefix, and sums the values
// down to it; a window with an unpublished entry before that is re-read
// (bounded: kSpinLimit rounds, then kErrTimeout).
__device__ uint32_t tile_prefix(uint32_t* tile_state, uint32_t tile, uint32_t count) {
    __shared__ uint32_t s_prefix;
    if (threadIdx.x < 32) {
        const uint32_t lane = threadIdx.x;
        if (tile == 0) {
            if (lane == 0) {
                atomicExch(&tile_state[0], kFlagPrefix | count);
                s_prefix = 0;
            }
        } else {
            if (lane == 0) atomicExch(&tile_state[tile], kFlagAggregate | count);
            uint32_t excl = 0, spins = 0;
            int32_t top = (int32_t)tile - 1;
            for (;;) {
                const int32_t t = top - (int32_t)lane;
                // Below tile 0: a virtual inclusive prefix of 0.
                uint32_t st = kFlagPrefix;
                if (t >= 0) st = *((volatile uint32_t*)&tile_state[t]);
                const uint32_t flag = st & ~kValueMask;
                const uint32_t pref = __ballot_sync(0xffffffffu, flag == kFlagPrefix);
                const uint32_t unset = __ballot_sync(0xffffffffu, flag == 0u);
                const uint32_t p = pref ? (uint32_t)__ffs(pref) - 1u : 32u;
                const uint32_t upto = p < 31u ? ((2u << p) - 1u) : 0xffffffffu;  // lanes 0..p
                if (unset & upto) {
                    if (++spins > kSpinLimit) {
                        raise_status(kErrTimeout);
                        break;
                    }
                    continue;
                }
                excl += __reduce_add_sync(0xffffffffu, lane <= p ? (st & kValueMask) : 0u);
                if (p < 32u) break;
                top -= 32;
            }
            if (lane == 0) {
                atomicExch(&tile_state[tile], kFlagPrefix | (excl + count));
                s_prefix = excl;
            }
        }
    }
    __syncthreads();
    return s_prefix;
}

// raygenPath.comp:95-167.  scratch[0] = tile ticket, scratch[1..] = tile
// states; both zeroed by the host before the launch.  MK >= 0: also writes
// the Morton key of kind MK of every output ray and its index (keys[dst],
// key_idx[dst] = dst), which the Morton kernel would otherwise compute
// from the written rays.
template <int MK>
__global__ void k_raygen_path(uint32_t* __restrict__ seeds, const wfpt_geometry* __restrict__ geoms,
                              const float4* __restrict__ in_rays, float4* __restrict__ out_rays,
                              const int32_t* __restrict__ in_i2p, int32_t* __restrict__ out_i2p,
                              const int4* __restrict__ in_results, float4* __restrict__ decreases,
                              uint32_t* __restrict__ out_count, uint32_t n,
                              const uint32_t* __restrict__ n_dev, float albedo,
                              uint32_t* __restrict__ scratch, void* __restrict__ keys,
                              uint32_t* __restrict__ key_idx, Box6 box) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kBlock / 32];
    uint32_t count = load_count(n, n_dev);
    uint32_t ntiles = (count + kBlock - 1) / kBlock;
    if (threadIdx.x == 0) s_tile = atomicAdd(&scratch[0], 1u);
    __syncthreads();
    uint32_t tile = s_tile;
    if (ntiles == 0) {
        if (tile == 0 && threadIdx.x == 0) *out_count = 0;
        return;
    }
    if (tile >= ntiles) return;
    uint32_t task = tile * kBlock + threadIdx.x;
    bool active = false;
    float4 o0 = make_float4(0, 0, 0, 0), o1 = o0, dc = o0;
    int pixel = 0;
    if (task < count) {
        pixel = in_i2p[task];
        uint32_t seed = seeds[task];
        int4 res = in_results[task];
        if (res.x >= 0) {
            float4 r0 = in_rays[2 * task + 0];
            float4 r1 = in_rays[2 * task + 1];
            f3 dir = mk(r1.x, r1.y, r1.z);
            f3 nrm = unpack_normal(geoms, res.y, res.x, (uint32_t)res.w);
            f3 ff = faceforward(nrm, dir, nrm);
            float ra = randf(seed);
            float rb = randf(seed);
            float t = __int_as_float(res.z);
            f3 hit = add(mk(r0.x, r0.y, r0.z), mul(dir, t));
            const float EPS = 1.0e-4f;
            f3 nd = cosine_random_vector(ra, rb, ff);
            f3 org = add(hit, mul(nd, EPS));
            o0 = make_float4(org.x, org.y, org.z, EPS);
            o1 = make_float4(nd.x, nd.y, nd.z, 3.402823466e+38f);
            active = true;
            seeds[task] = seed;
            // Read the pixel's path throughput now (each pixel has one ray
            // per pass): the load overlaps the look-back below instead of
            // following it (12 % faster at the frame's 2.07M rays).
            dc = decreases[pixel];
        }
    }
    // Block-level ordered ranks.
    uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t ballot = __ballot_sync(0xffffffffu, active);
    uint32_t lane_rank = __popc(ballot & ((1u << lane) - 1u));
    if (lane == 0) s_warp[warp] = __popc(ballot);
    __syncthreads();
    uint32_t warp_off = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kBlock / 32; ++w) {
        uint32_t c = s_warp[w];
        if (w < (int)warp) warp_off += c;
        total += c;
    }
    uint32_t base = tile_prefix(scratch + 1, tile, total);
    if (active && base + warp_off + lane_rank >= count) {  // only after a look-back timeout
        raise_status(kErrBounds);
        active = false;
    }
    if (active) {
        uint32_t dst = base + warp_off + lane_rank;
        out_rays[2 * dst + 0] = o0;
        out_rays[2 * dst + 1] = o1;
        out_i2p[dst] = pixel;
        if (MK >= 0) {
            write_morton_key<(MK < 0 ? 0 : MK)>(keys, dst, o0, o1, box);
            key_idx[dst] = dst;
        }
        dc.x = __fmul_rn(dc.x, albedo);
        dc.y = __fmul_rn(dc.y, albedo);
        dc.z = __fmul_rn(dc.z, albedo);
        dc.w = __fmul_rn(dc.w, 1.0f);
        decreases[pixel] = dc;
    }
    if (tile == ntiles - 1 && threadIdx.x == 0) *out_count = base + total;
}

// ---------------------------------------------------- reconstructSmooth
// reconstructSmooth.comp:44-94.  hit_count (nullable): also adds the
// number of hit records among the n rays to *hit_count, the count
// countRayHits.comp takes for the shadow pass that follows (same rays, same
// results), one atomic per block.  fresh != 0: the pixels of these rays
// are taken as zero instead of being read (the renderer's per-pass colour
// buffer, cleared before every pass in the reference: each of its pixels
// has one ray per pass), with the same addition to zero.
__global__ void k_reconstruct_smooth(const float4* __restrict__ rays, const int4* __restrict__ results,
                                     const int32_t* __restrict__ i2p, float4* __restrict__ pixels,
                                     const float4* __restrict__ decreases,
                                     const wfpt_geometry* __restrict__ geoms, float lx, float ly,
                                     float lz, float bx, float by, float bz, uint32_t n,
                                     const uint32_t* __restrict__ n_dev, int spp,
                                     uint32_t* __restrict__ hit_count, int fresh) {
    uint32_t task = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = task < load_count(n, n_dev);
    if (hit_count != nullptr) {
        __shared__ uint32_t s_w[kBlock / 32];
        const uint32_t c = __popc(__ballot_sync(0xffffffffu, valid && results[task].x >= 0));
        if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int w = 0; w < kBlock / 32; ++w) t += s_w[w];
            if (t) atomicAdd(hit_count, t);
        }
    }
    if (!valid) return;
    int pixel = i2p[task];
    const float4 pc = fresh ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : pixels[pixel];
    f3 color = mk(pc.x, pc.y, pc.z);
    float4 dc = decreases[pixel];
    f3 dec = mk(dc.x, dc.y, dc.z);
    int4 res = results[task];
    float fs = (float)spp;
    if (res.x == -1) {
        color = add(color, divs(mul(dec, mk(bx, by, bz)), fs));
    } else {
        float4 r0 = rays[2 * task + 0];
        float4 r1 = rays[2 * task + 1];
        f3 dir = mk(r1.x, r1.y, r1.z);
        f3 nrm = unpack_normal(geoms, res.y, res.x, (uint32_t)res.w);
        float t = __int_as_float(res.z);
        f3 hit = add(mk(r0.x, r0.y, r0.z), mul(dir, t));
        f3 L = normalize(sub(mk(lx, ly, lz), hit));
        f3 ff = faceforward(nrm, dir, nrm);
        float ndl = dot(ff, L);
        float alpha = fmaxf(ndl, 0.1f);
        color = add(color, divs(mul(dec, alpha), fs));
    }
    pixels[pixel] = make_float4(color.x, color.y, color.z, 1.0f);
}

// ---------------------------------------------------- reconstructShadow
// reconstructShadow.comp:39-59.
__global__ void k_reconstruct_shadow(const int4* __restrict__ results, const int32_t* __restrict__ i2p,
                                     const int32_t* __restrict__ i2s,
                                     const float4* __restrict__ in_pixels, float4* __restrict__ out_pixels,
                                     int batch_begin, int batch_size,
                                     const uint32_t* __restrict__ n_in_dev, int S, int replace) {
    uint32_t task = blockIdx.x * blockDim.x + threadIdx.x;
    int size = batch_size;
    if (n_in_dev != nullptr) {
        int avail = (int)*n_in_dev - batch_begin;
        if (avail < size) size = avail;
    }
    if ((int)task >= size) return;
    int pixel = i2p[batch_begin + task];
    float4 ip = in_pixels[pixel];
    float shadow = 0.0f;
    for (int i = 0; i < S; ++i) {
        int slot = i2s[(int)task * S + i];
        if (results[slot].x == -1) shadow = __fadd_rn(shadow, 1.0f);
    }
    shadow = __fdiv_rn(shadow, (float)S);
    float4 c = make_float4(__fmul_rn(ip.x, shadow), __fmul_rn(ip.y, shadow), __fmul_rn(ip.z, shadow), 1.0f);
    if (replace) {
        out_pixels[pixel] = c;
    } else {
        float4 o = out_pixels[pixel];
        out_pixels[pixel] =
            make_float4(__fadd_rn(o.x, c.x), __fadd_rn(o.y, c.y), __fadd_rn(o.z, c.z), __fadd_rn(o.w, c.w));
    }
}

// --------------------------------------------------------- countRayHits
// countRayHits.comp:24-50 (warp reduce, block reduce, one atomic per block).
__global__ void k_count_hits(const int4* __restrict__ results, uint32_t n,
                             const uint32_t* __restrict__ n_dev, uint32_t* __restrict__ count) {
    __shared__ uint32_t s_w[kBlock / 32];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t c = (i < load_count(n, n_dev) && results[i].x >= 0) ? 1u : 0u;
    c = __popc(__ballot_sync(0xffffffffu, c != 0));
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kBlock / 32; ++w) t += s_w[w];
        if (t) atomicAdd(count, t);
    }
}

// ---------------------------------------------------- interpolateColors
// interpolateColors.comp:10-57 (Reinhard via RGB->XYZ->Yxy and back).
__device__ __forceinline__ f3 tonemap_reinhard(f3 c, float key, float white) {
    const float avg_lum = 0.5f;
    float X = __fadd_rn(__fadd_rn(__fmul_rn(0.5141364f, c.x), __fmul_rn(0.265068f, c.y)), __fmul_rn(0.0241188f, c.z));
    float Y = __fadd_rn(__fadd_rn(__fmul_rn(0.3238786f, c.x), __fmul_rn(0.67023428f, c.y)), __fmul_rn(0.1228178f, c.z));
    float Z = __fadd_rn(__fadd_rn(__fmul_rn(0.16036376f, c.x), __fmul_rn(0.06409157f, c.y)), __fmul_rn(0.84442666f, c.z));
    float sum = __fadd_rn(__fadd_rn(X, Y), Z);
    float yl = Y;
    float xx = __fdiv_rn(X, sum);
    float yy = __fdiv_rn(Y, sum);
    float lp = __fdiv_rn(__fmul_rn(yl, key), avg_lum);
    float ld = __fdiv_rn(__fmul_rn(lp, __fadd_rn(1.0f, __fdiv_rn(lp, __fmul_rn(white, white)))), __fadd_rn(1.0f, lp));
    float X2 = __fdiv_rn(__fmul_rn(ld, xx), yy);
    float Y2 = ld;
    float Z2 = __fdiv_rn(__fmul_rn(ld, __fsub_rn(__fsub_rn(1.0f, xx), yy)), yy);
    f3 o;
    o.x = __fadd_rn(__fadd_rn(__fmul_rn(2.5651f, X2), __fmul_rn(-1.0217f, Y2)), __fmul_rn(0.0753f, Z2));
    o.y = __fadd_rn(__fadd_rn(__fmul_rn(-1.1665f, X2), __fmul_rn(1.9777f, Y2)), __fmul_rn(-0.2543f, Z2));
    o.z = __fadd_rn(__fadd_rn(__fmul_rn(-0.3986f, X2), __fmul_rn(0.0439f, Y2)), __fmul_rn(1.1892f, Z2));
    return o;
}

// interpolateColors.comp:78-97.
__global__ void k_interpolate_colors(float4* __restrict__ frame_pixels, float4* __restrict__ pixels,
                                     uint32_t n, int frame_index, float key, float white,
                                     const FrameParams* __restrict__ fp) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (fp) frame_index = fp->frame_index;
    if (frame_index > 1) {
        float4 p0 = pixels[i];
        float4 p1 = frame_pixels[i];
        float a = __fdiv_rn(1.0f, (float)frame_index);
        float b = __fmul_rn(a, __fsub_rn((float)frame_index, 1.0f));
        f3 c = add(mul(mk(p1.x, p1.y, p1.z), a), mul(mk(p0.x, p0.y, p0.z), b));
        pixels[i] = make_float4(c.x, c.y, c.z, 1.0f);
        f3 t = tonemap_reinhard(c, key, white);
        frame_pixels[i] = make_float4(t.x, t.y, t.z, 1.0f);
    } else {
        float4 c = frame_pixels[i];
        pixels[i] = c;
        f3 t = tonemap_reinhard(mk(c.x, c.y, c.z), key, white);
        frame_pixels[i] = make_float4(t.x, t.y, t.z, 1.0f);
    }
}

// interpolateColors.comp:78-97 with the running mean kept in double: the
// frame's colour (frame_pixels, float) is blended into accum (double4 per
// pixel, w unused) with a = 1/frame and b = a * (frame - 1) in double, one
// rounding per operation; pixels receives the mean rounded to float (w: the
// frame colour's w on frame 1, 1 later, as the shader), and the tone map
// (in float, as the shader) reads that rounding.
__device__ __forceinline__ double dblend(double c1, double c0, double a, double b) {
    return __dadd_rn(__dmul_rn(a, c1), __dmul_rn(b, c0));
}

__global__ void k_interpolate_colors_fp64(float4* __restrict__ frame_pixels, float4* __restrict__ pixels,
                                          double4_32a* __restrict__ accum, uint32_t n, int frame_index, float key,
                                          float white, const FrameParams* __restrict__ fp) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (fp) frame_index = fp->frame_index;
    float4 p1 = frame_pixels[i];
    double4_32a m;
    if (frame_index > 1) {
        double4_32a m0 = accum[i];
        double a = __ddiv_rn(1.0, (double)frame_index);
        double b = __dmul_rn(a, __dsub_rn((double)frame_index, 1.0));
        m = make_double4_32a(dblend(p1.x, m0.x, a, b), dblend(p1.y, m0.y, a, b), dblend(p1.z, m0.z, a, b), 1.0);
    } else {
        m = make_double4_32a(p1.x, p1.y, p1.z, 1.0);
    }
    accum[i] = m;
    f3 c = mk(__double2float_rn(m.x), __double2float_rn(m.y), __double2float_rn(m.z));
    pixels[i] = make_float4(c.x, c.y, c.z, frame_index > 1 ? 1.0f : p1.w);
    f3 t = tonemap_reinhard(c, key, white);
    frame_pixels[i] = make_float4(t.x, t.y, t.z, 1.0f);
}

// Device-side size of one shadow batch: S * clamp(n_in - begin, 0, size).
__global__ void k_batch_count(const uint32_t* __restrict__ n_in_dev, uint32_t begin, uint32_t size, uint32_t S,
                              uint32_t* __restrict__ out) {
    uint32_t n_in = *n_in_dev;
    uint32_t avail = n_in > begin ? n_in - begin : 0u;
    *out = S * (avail < size ? avail : size);
}

__global__ void k_fill_u32(uint32_t* __restrict__ dst, uint32_t v, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) dst[i] = v;
}

// ------------------------------------------------------------ launchers
static inline unsigned grid_for(uint64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

cudaError_t launch_init_seeds(uint32_t* seeds, uint32_t n, int frame, cudaStream_t s, const FrameParams* fp) {
    if (n == 0) return cudaSuccess;
    k_init_seeds<<<grid_for(n), kBlock, 0, s>>>(seeds, n, (uint32_t)frame, fp);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_raygen_primary(const float* m, const int32_t* i2p, wfpt_ray* rays, const float* o,
                                  int sample_index, int w, int h, float max_dist, cudaStream_t s,
                                  const FrameParams* fp, int pass, int spp) {
    uint64_t n = (uint64_t)w * (uint64_t)h;
    if (n == 0) return cudaSuccess;
    Mat4 mm;
    for (int i = 0; i < 16; ++i) mm.m[i] = m ? m[i] : 0.0f;
    float oo[3] = {o ? o[0] : 0.0f, o ? o[1] : 0.0f, o ? o[2] : 0.0f};
    k_raygen_primary<<<grid_for(n), kBlock, 0, s>>>(mm, i2p, reinterpret_cast<float4*>(rays), oo[0], oo[1],
                                                    oo[2], sample_index, w, h, max_dist, fp, pass, spp);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_raygen_shadow(const uint32_t* seeds, const wfpt_ray* in_rays, const wfpt_hit* in_res,
                                 wfpt_ray* out_rays, int32_t* s2i, int32_t* i2s, const float* light,
                                 float radius, int bb, int bs, const uint32_t* n_in_dev, int S,
                                 cudaStream_t s) {
    if (bs <= 0) return cudaSuccess;
    k_raygen_shadow<<<grid_for((uint64_t)bs), kBlock, 0, s>>>(
        seeds, reinterpret_cast<const float4*>(in_rays), reinterpret_cast<const int4*>(in_res),
        reinterpret_cast<float4*>(out_rays), s2i, i2s, light[0], light[1], light[2], radius, bb, bs,
        n_in_dev, S);
    count_launch();
    return cudaGetLastError();
}

size_t raygen_path_scratch_bytes(uint32_t max_n) {
    size_t tiles = ((size_t)max_n + kBlock - 1) / kBlock;
    return (1 + tiles + 1) * sizeof(uint32_t);
}

cudaError_t launch_raygen_path(uint32_t* seeds, const wfpt_geometry* geoms, const wfpt_ray* in_rays,
                               wfpt_ray* out_rays, const int32_t* in_i2p, int32_t* out_i2p,
                               const wfpt_hit* in_res, float* decreases, uint32_t* out_count,
                               uint32_t n, const uint32_t* n_dev, float albedo, void* scratch,
                               cudaStream_t s, const MortonOut* mo) {
    size_t tiles = ((size_t)n + kBlock - 1) / kBlock;
    cudaError_t e = cudaMemsetAsync(scratch, 0, (1 + tiles) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    unsigned grid = tiles == 0 ? 1u : (unsigned)tiles;
    const Box6 box = mo ? mo->box : Box6{};
    auto k = k_raygen_path<-1>;
    if (mo != nullptr) {
        k = mo->kind == WFPT_MORTON_AILA32 ? k_raygen_path<WFPT_MORTON_AILA32>
            : mo->kind == WFPT_MORTON_6D48 ? k_raygen_path<WFPT_MORTON_6D48>
                                           : k_raygen_path<WFPT_MORTON_6D64>;
    }
    k<<<grid, kBlock, 0, s>>>(seeds, geoms, reinterpret_cast<const float4*>(in_rays),
                              reinterpret_cast<float4*>(out_rays), in_i2p, out_i2p,
                              reinterpret_cast<const int4*>(in_res), reinterpret_cast<float4*>(decreases),
                              out_count, n, n_dev, albedo, reinterpret_cast<uint32_t*>(scratch),
                              mo ? mo->keys : nullptr, mo ? mo->indices : nullptr, box);
    count_launch();
    return cudaGetLastError();
}

// Failure-detection self-test: the path compaction over two 256-ray tiles
// of misses, run by a single block that draws ticket 1, so its look-back
// waits on tile 0, which nothing publishes; the wait gives up after
// kSpinLimit rounds and latches kErrTimeout.  All rays miss, so nothing but
// the count is written.  Synchronises the stream.
cudaError_t raygen_path_selftest_timeout(cudaStream_t s) {
    constexpr uint32_t N = 2 * kBlock;
    // seeds, i2p in/out, count, scratch (ticket + 2 tile states) as words;
    // rays in/out, results, decreases as 16-byte records.
    const size_t words = 3 * (size_t)N + 1 + 3;
    const size_t vec4s = 2 * (size_t)N * 2 + N + N;
    unsigned char* buf = nullptr;
    cudaError_t e = dev_malloc(reinterpret_cast<void**>(&buf), vec4s * 16 + words * 4);
    if (e != cudaSuccess) return e;
    float4* in_rays = reinterpret_cast<float4*>(buf);
    float4* out_rays = in_rays + 2 * N;
    int4* results = reinterpret_cast<int4*>(out_rays + 2 * N);
    float4* decreases = reinterpret_cast<float4*>(results + N);
    uint32_t* seeds = reinterpret_cast<uint32_t*>(decreases + N);
    int32_t* in_i2p = reinterpret_cast<int32_t*>(seeds + N);
    int32_t* out_i2p = in_i2p + N;
    uint32_t* count = reinterpret_cast<uint32_t*>(out_i2p + N);
    uint32_t* scratch = count + 1;
    const uint32_t one = 1;
    e = cudaMemsetAsync(buf, 0, vec4s * 16 + words * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(results, 0xFF, N * sizeof(int4), s);  // every ray a miss
    if (e == cudaSuccess) e = cudaMemcpyAsync(scratch, &one, sizeof(one), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        k_raygen_path<-1><<<1, kBlock, 0, s>>>(seeds, nullptr, in_rays, out_rays, in_i2p, out_i2p, results,
                                               decreases, count, N, nullptr, 0.8f, scratch, nullptr, nullptr,
                                               Box6{});
        count_launch();
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(buf);
    return e != cudaSuccess ? e : e2;
}

// Library-owned compaction scratch for launch_raygen_path_static: the tile
// ticket (word 0) and one look-back state per 256-ray tile (words 1..),
// for at most WFPT_RAYGEN_PATH_STATIC_MAX_RAYS rays; 65,537 words (256 KiB)
// per device, placed by the module loader, never by an allocation call.
constexpr size_t kPathStaticWords = 1 + (WFPT_RAYGEN_PATH_STATIC_MAX_RAYS + kBlock - 1) / kBlock;
static __device__ __align__(256) uint32_t g_path_static_scratch[kPathStaticWords];

namespace {
// Device addresses of g_path_static_scratch, one per CUDA context, keyed by
// the context's unique id (cuCtxGetId: never reused within a process, so an
// entry left by a context that was destroyed, for example by
// cudaDeviceReset, can never match a later one).  The driver entry points
// are resolved through the runtime, so the library does not link libcuda.
struct StaticScratchEntry {
    unsigned long long ctx_id;
    uint32_t* ptr;
};
constexpr int kStaticScratchEntries = 64;
std::mutex g_path_static_mu;
StaticScratchEntry g_path_static_cache[kStaticScratchEntries] = {};
int g_path_static_next = 0;
PFN_cuCtxGetCurrent_v4000 g_cu_ctx_get_current = nullptr;
PFN_cuCtxGetId_v12000 g_cu_ctx_get_id = nullptr;

cudaError_t resolve_ctx_entry_points() {
    if (g_cu_ctx_get_current && g_cu_ctx_get_id) return cudaSuccess;
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault, &q1);
    if (e != cudaSuccess) return e;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess) return e;
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
        return cudaErrorSymbolNotFound;
    g_cu_ctx_get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f1);
    g_cu_ctx_get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f2);
    return cudaSuccess;
}

// Unique id of the context current on this thread; false when none is.
bool current_ctx_id(unsigned long long* id) {
    CUcontext ctx = nullptr;
    if (g_cu_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return g_cu_ctx_get_id(ctx, id) == CUDA_SUCCESS;
}

// Device address of g_path_static_scratch in the current context.  The
// first call in a context looks it up with cudaGetSymbolAddress (which may
// load the module); that first call is refused while `s` is capturing,
// with cudaErrorStreamCaptureUnsupported, so that no lookup runs inside a
// capture.  Later calls in the same context only read the cache.
cudaError_t path_static_scratch(uint32_t** out, cudaStream_t s) {
    std::lock_guard<std::mutex> lock(g_path_static_mu);
    cudaError_t e = resolve_ctx_entry_points();
    if (e != cudaSuccess) return e;
    unsigned long long id = 0;
    if (current_ctx_id(&id)) {
        for (const StaticScratchEntry& c : g_path_static_cache)
            if (c.ptr && c.ctx_id == id) {
                *out = c.ptr;
                return cudaSuccess;
            }
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess) return e;
    if (cap != cudaStreamCaptureStatusNone) return cudaErrorStreamCaptureUnsupported;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_path_static_scratch);
    if (e != cudaSuccess) return e;
    if (!current_ctx_id(&id)) return cudaErrorDeviceUninitialized;
    g_path_static_cache[g_path_static_next] = StaticScratchEntry{id, static_cast<uint32_t*>(p)};
    g_path_static_next = (g_path_static_next + 1) % kStaticScratchEntries;
    *out = static_cast<uint32_t*>(p);
    return cudaSuccess;
}
}  // namespace

cudaError_t launch_raygen_path_static(uint32_t* seeds, const wfpt_geometry* geoms, const wfpt_ray* in_rays,
                                      wfpt_ray* out_rays, const int32_t* in_i2p, int32_t* out_i2p,
                                      const wfpt_hit* in_res, float* decreases, uint32_t* out_count,
                                      uint32_t n, const uint32_t* n_dev, float albedo, cudaStream_t s) {
    if (n > WFPT_RAYGEN_PATH_STATIC_MAX_RAYS) return cudaErrorInvalidValue;
    uint32_t* scratch = nullptr;
    cudaError_t e = path_static_scratch(&scratch, s);
    if (e != cudaSuccess) return e;
    // The ticket and the tile states of this call's tiles start at zero.
    size_t tiles = ((size_t)n + kBlock - 1) / kBlock;
    e = cudaMemsetAsync(scratch, 0, (1 + tiles) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    unsigned grid = tiles == 0 ? 1u : (unsigned)tiles;
    k_raygen_path<-1><<<grid, kBlock, 0, s>>>(
        seeds, geoms, reinterpret_cast<const float4*>(in_rays), reinterpret_cast<float4*>(out_rays), in_i2p,
        out_i2p, reinterpret_cast<const int4*>(in_res), reinterpret_cast<float4*>(decreases), out_count, n,
        n_dev, albedo, scratch, nullptr, nullptr, Box6{});
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_reconstruct_smooth(const wfpt_ray* rays, const wfpt_hit* res, const int32_t* i2p,
                                      float* pixels, const float* decreases, const wfpt_geometry* geoms,
                                      const float* light, const float* bg, uint32_t n,
                                      const uint32_t* n_dev, int spp, cudaStream_t s, uint32_t* hit_count,
                                      bool fresh) {
    if (n == 0) return cudaSuccess;
    k_reconstruct_smooth<<<grid_for(n), kBlock, 0, s>>>(
        reinterpret_cast<const float4*>(rays), reinterpret_cast<const int4*>(res), i2p,
        reinterpret_cast<float4*>(pixels), reinterpret_cast<const float4*>(decreases), geoms, light[0],
        light[1], light[2], bg[0], bg[1], bg[2], n, n_dev, spp, hit_count, fresh ? 1 : 0);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_reconstruct_shadow(const wfpt_hit* res, const int32_t* i2p, const int32_t* i2s,
                                      const float* in_pixels, float* out_pixels, int bb, int bs,
                                      const uint32_t* n_in_dev, int S, int replace, cudaStream_t s) {
    if (bs <= 0) return cudaSuccess;
    k_reconstruct_shadow<<<grid_for((uint64_t)bs), kBlock, 0, s>>>(
        reinterpret_cast<const int4*>(res), i2p, i2s, reinterpret_cast<const float4*>(in_pixels),
        reinterpret_cast<float4*>(out_pixels), bb, bs, n_in_dev, S, replace);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_count_hits(const wfpt_hit* res, uint32_t n, const uint32_t* n_dev, uint32_t* count,
                              cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_count_hits<<<grid_for(n), kBlock, 0, s>>>(reinterpret_cast<const int4*>(res), n, n_dev, count);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_interpolate_colors(float* frame_pixels, float* pixels, uint32_t n, int frame_index,
                                      float key, float white, cudaStream_t s, const FrameParams* fp) {
    if (n == 0) return cudaSuccess;
    k_interpolate_colors<<<grid_for(n), kBlock, 0, s>>>(reinterpret_cast<float4*>(frame_pixels),
                                                        reinterpret_cast<float4*>(pixels), n, frame_index,
                                                        key, white, fp);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_interpolate_colors_fp64(float* frame_pixels, float* pixels, double* accum, uint32_t n,
                                           int frame_index, float key, float white, cudaStream_t s,
                                           const FrameParams* fp) {
    if (n == 0) return cudaSuccess;
    k_interpolate_colors_fp64<<<grid_for(n), kBlock, 0, s>>>(reinterpret_cast<float4*>(frame_pixels),
                                                             reinterpret_cast<float4*>(pixels),
                                                             reinterpret_cast<double4_32a*>(accum), n, frame_index, key,
                                                             white, fp);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_batch_count(const uint32_t* n_in_dev, uint32_t begin, uint32_t size, int S, uint32_t* out,
                               cudaStream_t s) {
    k_batch_count<<<1, 1, 0, s>>>(n_in_dev, begin, size, (uint32_t)S, out);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_fill_u32(void* dst, uint32_t v, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    size_t g = (n + kBlock - 1) / kBlock;
    unsigned grid = (unsigned)(g > 152 * 16 ? 152 * 16 : g);
    k_fill_u32<<<grid, kBlock, 0, s>>>(reinterpret_cast<uint32_t*>(dst), v, n);
    count_launch();
    return cudaGetLastError();
}

}  // namespace wfpt
