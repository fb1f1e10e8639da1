// Morton key generation and the ray-reorder gather.
//
// Both are HBM-bound streaming kernels: Morton reads one 32-byte ray and
// writes a key (4 or 8 B) plus an index (4 B); reorder gathers one 32-byte
// ray and one slot-map entry by the sorted permutation, writes them in
// order and scatters the inverse slot map.
#include "common.cuh"
#include "morton.cuh"
#include "stages.cuh"

namespace wfpt {

template <int KIND>
__global__ void k_morton(const float4* __restrict__ rays, uint32_t n, const uint32_t* __restrict__ n_dev,
                         Box6 box, void* __restrict__ keys, uint32_t* __restrict__ indices) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= load_count(n, n_dev)) return;
    float4 r0 = rays[2 * i + 0];
    float4 r1 = rays[2 * i + 1];
    write_morton_key<KIND>(keys, i, r0, r1, box);
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
