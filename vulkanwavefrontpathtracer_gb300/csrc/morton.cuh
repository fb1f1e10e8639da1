// Morton keys of ray records (computeMortonCodesAila32.comp and the 6-D
// kinds), shared by the Morton kernel and the path-ray generation that
// writes the keys of the rays it creates.
#pragma once

#include "common.cuh"
#include "stages.cuh"

namespace wfpt {

// computeMortonCodesAila32.comp:39-43: normalised origin in the scene box
// and the direction mapped to [0,1]^3.
__device__ __forceinline__ void morton_point(const float4& r0, const float4& r1, const float* smin,
                                             const float* ssize, f3& a, f3& b) {
    f3 o = mk(r0.x, r0.y, r0.z);
    f3 rel = divs3(sub(o, mk(smin[0], smin[1], smin[2])), mk(ssize[0], ssize[1], ssize[2]));
    a = mk(fminf(fmaxf(rel.x, 0.0f), 1.0f), fminf(fmaxf(rel.y, 0.0f), 1.0f), fminf(fmaxf(rel.z, 0.0f), 1.0f));
    f3 n = normalize(mk(r1.x, r1.y, r1.z));
    b = mk(__fmul_rn(__fadd_rn(n.x, 1.0f), 0.5f), __fmul_rn(__fadd_rn(n.y, 1.0f), 0.5f),
           __fmul_rn(__fadd_rn(n.z, 1.0f), 0.5f));
}

__device__ __forceinline__ uint32_t quant(float v, float scale) { return __float2uint_rz(__fmul_rn(v, scale)); }

// computeMortonCodesAila32.comp:42-88: 7 bits per origin axis, 4 bits per
// direction axis; bit layout (MSB first) ia6 ia5 ia4 ia3 ib3 ia2 ib2 ia1
// ib1 ia0 ib0(x,y only), each group as x y z.
__device__ __forceinline__ uint32_t aila32(uint32_t ax, uint32_t ay, uint32_t az, uint32_t bx, uint32_t by,
                                           uint32_t bz) {
    uint32_t k = 0;
#pragma unroll
    for (int l = 6; l >= 3; --l) {
        int p = 20 + 3 * (l - 3);
        k |= ((ax >> l) & 1u) << (p + 2);
        k |= ((ay >> l) & 1u) << (p + 1);
        k |= ((az >> l) & 1u) << p;
    }
    k |= ((bx >> 3) & 1u) << 19; k |= ((by >> 3) & 1u) << 18; k |= ((bz >> 3) & 1u) << 17;
    k |= ((ax >> 2) & 1u) << 16; k |= ((ay >> 2) & 1u) << 15; k |= ((az >> 2) & 1u) << 14;
    k |= ((bx >> 2) & 1u) << 13; k |= ((by >> 2) & 1u) << 12; k |= ((bz >> 2) & 1u) << 11;
    k |= ((ax >> 1) & 1u) << 10; k |= ((ay >> 1) & 1u) << 9;  k |= ((az >> 1) & 1u) << 8;
    k |= ((bx >> 1) & 1u) << 7;  k |= ((by >> 1) & 1u) << 6;  k |= ((bz >> 1) & 1u) << 5;
    k |= ((ax >> 0) & 1u) << 4;  k |= ((ay >> 0) & 1u) << 3;  k |= ((az >> 0) & 1u) << 2;
    k |= ((bx >> 0) & 1u) << 1;  k |= ((by >> 0) & 1u) << 0;
    return k;
}

// Moves bit i of an 11-bit value to bit 6i (shifts 40/20/10/5 selected by
// the binary digits of i).
__device__ __forceinline__ uint64_t spread6(uint64_t x) {
    x &= 0x7FFull;
    x = (x | (x << 40)) & 0x00070000000000FFull;
    x = (x | (x << 20)) & 0x000700000F00000Full;
    x = (x | (x << 10)) & 0x1003003003003003ull;
    x = (x | (x << 5)) & 0x1041041041041041ull;
    return x;
}

// 6-D keys: per bit level l the six bits ox oy oz dx dy dz at positions
// 6l+5 .. 6l.  WFPT_MORTON_6D48: 8 bits per axis, levels 0..7 (48 bits).
// WFPT_MORTON_6D64: origin 11 bits, direction 10 bits; levels 0..9 as
// above and the origin's bit 10 at positions 62 (x), 61 (y), 60 (z).
__device__ __forceinline__ uint64_t key6d(uint32_t ax, uint32_t ay, uint32_t az, uint32_t bx, uint32_t by,
                                          uint32_t bz) {
    uint64_t k = (spread6(ax & 0x3FFu) << 5) | (spread6(ay & 0x3FFu) << 4) | (spread6(az & 0x3FFu) << 3) |
                 (spread6(bx) << 2) | (spread6(by) << 1) | spread6(bz);
    k |= (uint64_t)((ax >> 10) & 1u) << 62;
    k |= (uint64_t)((ay >> 10) & 1u) << 61;
    k |= (uint64_t)((az >> 10) & 1u) << 60;
    return k;
}

// Key KIND of ray record (r0, r1) in the scene box, written at keys[i].
template <int KIND>
__device__ __forceinline__ void write_morton_key(void* __restrict__ keys, uint32_t i, const float4& r0,
                                                 const float4& r1, const Box6& box) {
    f3 a, b;
    morton_point(r0, r1, box.smin, box.ssize, a, b);
    if (KIND == WFPT_MORTON_AILA32) {
        uint32_t k = aila32(quant(a.x, 127.0f), quant(a.y, 127.0f), quant(a.z, 127.0f), quant(b.x, 15.0f),
                            quant(b.y, 15.0f), quant(b.z, 15.0f));
        reinterpret_cast<uint32_t*>(keys)[i] = k;
    } else if (KIND == WFPT_MORTON_6D48) {
        uint64_t k = key6d(quant(a.x, 255.0f), quant(a.y, 255.0f), quant(a.z, 255.0f), quant(b.x, 255.0f),
                           quant(b.y, 255.0f), quant(b.z, 255.0f));
        reinterpret_cast<uint64_t*>(keys)[i] = k;
    } else {
        uint64_t k = key6d(quant(a.x, 2047.0f), quant(a.y, 2047.0f), quant(a.z, 2047.0f), quant(b.x, 1023.0f),
                           quant(b.y, 1023.0f), quant(b.z, 1023.0f));
        reinterpret_cast<uint64_t*>(keys)[i] = k;
    }
}

}  // namespace wfpt
