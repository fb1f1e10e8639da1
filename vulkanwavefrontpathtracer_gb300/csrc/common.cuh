// Shared device-side definitions for the wavefront stage kernels.
//
// Float arithmetic in the shading and key-generation kernels is written with
// explicit round-to-nearest intrinsics (__fmul_rn, __fadd_rn, ...) so that
// nvcc never contracts a*b+c into an FMA.  The CPU oracle evaluates the same
// operations in the same order with -ffp-contract=off, which makes these
// kernels bit-exact against it on every input.  Traversal uses the same
// discipline for the ray/triangle test (watertightness needs it anyway).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/wfpt.h"

namespace wfpt {

static_assert(sizeof(wfpt_ray) == 32, "Ray record must be 32 bytes (Ray.h:32-37)");
static_assert(sizeof(wfpt_hit) == 16, "RayResult record must be 16 bytes (Ray.h:39-44)");
static_assert(sizeof(wfpt_geometry) == 16, "Geometry record must be 16 bytes");

constexpr int kBlock = 256;  // THREADBLOCK_SIZE of every reference shader

// Device status word bits (read by wfpt_device_status).
constexpr uint32_t kErrTimeout = 1u;
constexpr uint32_t kErrBounds = 2u;

// Bounded spin budget for decoupled look-back waits.  A predecessor tile
// that never publishes makes the waiter give up after this many polls,
// latch kErrTimeout and continue, instead of hanging the GPU.
constexpr uint32_t kSpinLimit = 1u << 22;

// One status word per translation unit (no relocatable device code); each
// unit exports a reader that returns and clears it (see status_* below).
static __device__ uint32_t g_status = 0;

__device__ __forceinline__ void raise_status(uint32_t bits) { atomicOr(&g_status, bits); }

static inline cudaError_t read_and_clear_status(uint32_t* out) {
    uint32_t v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_status, sizeof(v));
    if (e != cudaSuccess) return e;
    *out |= v;
    if (v) {
        uint32_t z = 0;
        e = cudaMemcpyToSymbol(g_status, &z, sizeof(z));
    }
    return e;
}

__device__ __forceinline__ uint32_t load_count(uint32_t n, const uint32_t* n_dev) {
    if (n_dev == nullptr) return n;
    uint32_t d = *n_dev;
    return d < n ? d : n;
}

struct f3 {
    float x, y, z;
};

__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 add(f3 a, f3 b) {
    return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 sub(f3 a, f3 b) {
    return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 mul(f3 a, float s) {
    return {__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)};
}
__device__ __forceinline__ f3 mul(f3 a, f3 b) {
    return {__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 divs(f3 a, float s) {
    return {__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)};
}
__device__ __forceinline__ f3 divs3(f3 a, f3 b) {
    return {__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y), __fdiv_rn(a.z, b.z)};
}
// dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, no contraction.
__device__ __forceinline__ float dot(f3 a, f3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float length(f3 a) { return __fsqrt_rn(dot(a, a)); }
// normalize(a) = a / sqrt(dot(a,a)) with IEEE division and square root.
__device__ __forceinline__ f3 normalize(f3 a) { return divs(a, length(a)); }
// GLSL faceforward(N, I, Nref): dot(Nref, I) < 0 ? N : -N.
__device__ __forceinline__ f3 faceforward(f3 n, f3 i, f3 nref) {
    return dot(nref, i) < 0.0f ? n : mk(-n.x, -n.y, -n.z);
}

__device__ __forceinline__ f3 ld_origin(const float4& a) { return {a.x, a.y, a.z}; }

// Three-input minimum / maximum (one instruction on sm_100 and later);
// same NaN handling as fminf/fmaxf, and exact, so
// max3(a, b, c) == fmaxf(fmaxf(a, b), c) bit for bit.
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// GLSL packUnorm2x16 / unpackUnorm2x16.
__device__ __forceinline__ uint32_t pack_unorm2x16(float u, float v) {
    float cu = fminf(fmaxf(u, 0.0f), 1.0f);
    float cv = fminf(fmaxf(v, 0.0f), 1.0f);
    uint32_t a = (uint32_t)__float2int_rn(__fmul_rn(cu, 65535.0f));
    uint32_t b = (uint32_t)__float2int_rn(__fmul_rn(cv, 65535.0f));
    return a | (b << 16);
}
__device__ __forceinline__ void unpack_unorm2x16(uint32_t p, float& u, float& v) {
    u = __fdiv_rn((float)(p & 0xFFFFu), 65535.0f);
    v = __fdiv_rn((float)(p >> 16), 65535.0f);
}

// sin(2*pi*r) and cos(2*pi*r) for r in [0,1): quadrant reduction on 4r
// (exact in float for the 24-bit LCG samples), then Taylor series of sin
// to x^9 and cos to x^10 on |x| <= pi/4, evaluated by Horner with
// round-to-nearest operations.  Written from the series, so the CPU oracle
// evaluates the identical sequence.
__device__ __forceinline__ void sincos_2pi(float r, float& s, float& c) {
    float q4 = __fmul_rn(r, 4.0f);
    float q = rintf(q4);
    float f = __fsub_rn(q4, q);                      // [-0.5, 0.5]
    float x = __fmul_rn(f, 1.57079632679489662f);    // [-pi/4, pi/4]
    float x2 = __fmul_rn(x, x);
    // sin x = x(1 - x2/6 (1 - x2/20 (1 - x2/42 (1 - x2/72))))
    float ps = __fsub_rn(1.0f, __fmul_rn(x2, 1.0f / 72.0f));
    ps = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 1.0f / 42.0f), ps));
    ps = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 1.0f / 20.0f), ps));
    ps = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 1.0f / 6.0f), ps));
    float sx = __fmul_rn(x, ps);
    // cos x = 1 - x2/2 (1 - x2/12 (1 - x2/30 (1 - x2/56 (1 - x2/90))))
    float pc = __fsub_rn(1.0f, __fmul_rn(x2, 1.0f / 90.0f));
    pc = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 1.0f / 56.0f), pc));
    pc = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 1.0f / 30.0f), pc));
    pc = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 1.0f / 12.0f), pc));
    float cx = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 0.5f), pc));
    int quad = ((int)q) & 3;
    switch (quad) {
        case 0: s = sx; c = cx; break;
        case 1: s = cx; c = -sx; break;
        case 2: s = -sx; c = -cx; break;
        default: s = -cx; c = sx; break;
    }
}

}  // namespace wfpt
