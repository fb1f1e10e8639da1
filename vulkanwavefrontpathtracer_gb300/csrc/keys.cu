// Morton key generation and the ray-reorder gather.
//
// Both are HBM-bound streaming kernels: Morton reads one 32-byte ray and
// writes a key (4 or 8 B) plus an index (4 B); reorder gathers one 32-byte
// ray and one slot-map entry by the sorted permutation, writes them in
// order and scatters the inverse slot map.
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

struct Box6 {
    float smin[3];
    float ssize[3];
};

template <int KIND>
__global__ void k_morton(const float4* __restrict__ rays, uint32_t n, const uint32_t* __restrict__ n_dev,
                         Box6 box, void* __restrict__ keys, uint32_t* __restrict__ indices) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= load_count(n, n_dev)) return;
    float4 r0 = rays[2 * i + 0];
    float4 r1 = rays[2 * i + 1];
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
    indices[i] = i;
}

// Gathers beyond L2 (STREAM): the index, the gathered records and the
// written records are touched once, so they are loaded and stored with an
// L2 evict-first policy, and the L2 keeps the randomly accessed 4-byte slot
// map entries (each 32-byte sector of them is touched eight times, at random
// moments) for longer.  Random-permutation gathers of 32- / 48-byte records:
// 7 / 10 % faster at 2^22 rays, 26 / 20 % at 2^23, 9 / 6 % at 2^24, 2 % at
// 2^25; an evict-last policy on the slot maps instead was 3-12 % slower.
// Smaller gathers (a frame's 2.07M-ray wavefront, whose records the next
// kernel reads back from L2) keep plain accesses: the policy made 2^21 rays
// 5-10 % slower.
constexpr uint32_t kStreamRecords = 1u << 22;

__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
template <bool STREAM>
__device__ __forceinline__ uint4 load_record(const uint4* p, uint64_t pol) {
    if (!STREAM) return __ldg(p);
    uint4 v;
    asm volatile("ld.global.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}
template <bool STREAM>
__device__ __forceinline__ void store_record(uint4* p, uint4 v, uint64_t pol) {
    if (!STREAM) {
        *p = v;
        return;
    }
    asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "r"(v.x), "r"(v.y),
                 "r"(v.z), "r"(v.w), "l"(pol)
                 : "memory");
}

// reorderRays.comp:37-45.
template <bool STREAM>
__global__ void k_reorder(const uint32_t* __restrict__ idx, const uint4* __restrict__ in_rays,
                          uint4* __restrict__ out_rays, const int32_t* __restrict__ in_s2i,
                          int32_t* __restrict__ out_s2i, int32_t* __restrict__ out_i2s, uint32_t n,
                          const uint32_t* __restrict__ n_dev) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= load_count(n, n_dev)) return;
    const uint64_t pol = STREAM ? l2_evict_first_policy() : 0u;
    uint32_t old = STREAM ? __ldcs(idx + i) : idx[i];
    int32_t index = in_s2i[old];
    uint4 a = load_record<STREAM>(in_rays + 2 * (size_t)old + 0, pol);
    uint4 b = load_record<STREAM>(in_rays + 2 * (size_t)old + 1, pol);
    store_record<STREAM>(out_rays + 2 * (size_t)i + 0, a, pol);
    store_record<STREAM>(out_rays + 2 * (size_t)i + 1, b, pol);
    if (STREAM) {
        __stcs(out_s2i + i, index);
    } else {
        out_s2i[i] = index;
    }
    out_i2s[index] = (int32_t)i;
}

// The same gather for records of C x 16 bytes (ray records with a payload,
// 48 B = 3 chunks).  One thread per record: the C 16-byte loads of a record
// are issued together; stores are coalesced across the warp.  The slot maps
// are optional (in_s2i == nullptr: plain gather).
template <int C, bool STREAM>
__global__ void k_reorder_records(const uint32_t* __restrict__ idx, const uint4* __restrict__ in_rec,
                                  uint4* __restrict__ out_rec, const int32_t* __restrict__ in_s2i,
                                  int32_t* __restrict__ out_s2i, int32_t* __restrict__ out_i2s, uint32_t n,
                                  const uint32_t* __restrict__ n_dev) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= load_count(n, n_dev)) return;
    const uint64_t pol = STREAM ? l2_evict_first_policy() : 0u;
    uint32_t old = STREAM ? __ldcs(idx + i) : idx[i];
    uint4 v[C];
#pragma unroll
    for (int c = 0; c < C; ++c) v[c] = load_record<STREAM>(in_rec + (size_t)C * old + c, pol);
#pragma unroll
    for (int c = 0; c < C; ++c) store_record<STREAM>(out_rec + (size_t)C * i + c, v[c], pol);
    if (in_s2i != nullptr) {
        int32_t index = in_s2i[old];
        if (STREAM) {
            __stcs(out_s2i + i, index);
        } else {
            out_s2i[i] = index;
        }
        out_i2s[index] = (int32_t)i;
    }
}

cudaError_t launch_morton(const wfpt_ray* rays, uint32_t n, const uint32_t* n_dev, const float* smin,
                          const float* ssize, int kind, void* keys, uint32_t* indices, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    Box6 box;
    for (int k = 0; k < 3; ++k) {
        box.smin[k] = smin[k];
        box.ssize[k] = ssize[k];
    }
    unsigned grid = (n + kBlock - 1) / kBlock;
    const float4* r = reinterpret_cast<const float4*>(rays);
    switch (kind) {
        case WFPT_MORTON_AILA32: k_morton<WFPT_MORTON_AILA32><<<grid, kBlock, 0, s>>>(r, n, n_dev, box, keys, indices); break;
        case WFPT_MORTON_6D48: k_morton<WFPT_MORTON_6D48><<<grid, kBlock, 0, s>>>(r, n, n_dev, box, keys, indices); break;
        default: k_morton<WFPT_MORTON_6D64><<<grid, kBlock, 0, s>>>(r, n, n_dev, box, keys, indices); break;
    }
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_reorder(const uint32_t* idx, const wfpt_ray* in_rays, wfpt_ray* out_rays,
                           const int32_t* in_s2i, int32_t* out_s2i, int32_t* out_i2s, uint32_t n,
                           const uint32_t* n_dev, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    unsigned grid = (n + kBlock - 1) / kBlock;
    auto k = n >= kStreamRecords ? k_reorder<true> : k_reorder<false>;
    k<<<grid, kBlock, 0, s>>>(idx, reinterpret_cast<const uint4*>(in_rays), reinterpret_cast<uint4*>(out_rays), in_s2i,
                              out_s2i, out_i2s, n, n_dev);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_reorder_records(const uint32_t* idx, const void* in_records, void* out_records,
                                   uint32_t record_bytes, const int32_t* in_s2i, int32_t* out_s2i, int32_t* out_i2s,
                                   uint32_t n, const uint32_t* n_dev, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    unsigned grid = (n + kBlock - 1) / kBlock;
    const uint4* in = static_cast<const uint4*>(in_records);
    uint4* out = static_cast<uint4*>(out_records);
    const bool st = n >= kStreamRecords;
    switch (record_bytes) {
#define WFPT_REORDER_REC(B, C)                                                                                       \
    case B:                                                                                                          \
        (st ? k_reorder_records<C, true> : k_reorder_records<C, false>)<<<grid, kBlock, 0, s>>>(                     \
            idx, in, out, in_s2i, out_s2i, out_i2s, n, n_dev);                                                       \
        break;
        WFPT_REORDER_REC(16, 1) WFPT_REORDER_REC(32, 2) WFPT_REORDER_REC(48, 3) WFPT_REORDER_REC(64, 4)
#undef WFPT_REORDER_REC
        default: return cudaErrorInvalidValue;
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace wfpt
