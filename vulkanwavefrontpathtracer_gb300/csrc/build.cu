// Device build of the acceleration structures, for scenes that are large or
// already on the GPU.  Takes the place of the host builder (bvh.cpp; the
// reference's driver BLAS build, WaveFrontPathTracer.cpp:202-457):
//   1. triangle boxes, the centroid box and the largest absolute coordinate
//      (for the conservative box growth) in one pass;
//   2. 63-bit Morton keys of the triangle centroids, sorted with the
//      library's radix sort;
//   3. PLOC (Meister and Bittner, "Parallel Locally-Ordered Clustering for
//      Bounding Volume Hierarchy Construction", IEEE TVCG 2018): every
//      cluster picks the neighbour among the 8 (knob) on either side (in
//      Morton order) whose merged box has the least surface area, mutual pairs
//      merge, the cluster list is compacted by a prefix sum, until one
//      cluster is left;
//   4. the BVH2 in the traversal format (children's boxes grown by 2^-22 P
//      as in the host builder; single-triangle leaves);
//   5. the BVH8 by the host's SAH collapse: a bottom-up dynamic programme
//      (one thread per leaf climbs towards the root; the second thread to
//      arrive at a node computes it), then a top-down emission one level at
//      a time with prefix-summed allocation, so the layout is deterministic.
// Every loop over clusters or levels is bounded on the host; kernels check
// their indices against the buffers they write.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "build.cuh"
#include "common.cuh"
#include "scene.h"
#include "stages.cuh"

namespace wfpt {

cudaError_t status_build(uint32_t* out) { return read_and_clear_status(out); }

// PLOC search radius (clusters on either side in Morton order).  On the
// courtyard's bounce-1 rays 8 gave the fastest traversal of radii 8-64 (the
// BVH8 from radius 8 traced closest hits 8 % faster than from 16, 13 %
// faster than from 64).
static int g_ploc_radius = 8;
void set_ploc_radius(int r) { g_ploc_radius = r < 1 ? 1 : (r > 64 ? 64 : r); }
int get_ploc_radius() { return g_ploc_radius; }

namespace {

constexpr int kBB = 256;      // threads per build block
constexpr int kPlocRMax = 64;  // largest PLOC search radius (knob build.ploc.radius)
constexpr int kScanItems = 8;  // elements per thread of the prefix sum
constexpr uint32_t kNone = 0xFFFFFFFFu;

struct BuildStats {
    uint32_t bmin[3], bmax[3];  // order-preserving bits of the vertex box
    uint32_t cmin[3], cmax[3];  // ... of the centroid box
    uint32_t pmax;              // bits of the largest |coordinate|
    uint32_t bad_index;
};

__device__ __forceinline__ uint32_t ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__device__ __forceinline__ float box_area(float4 lo, float4 hi) {
    float dx = __fsub_rn(hi.x, lo.x), dy = __fsub_rn(hi.y, lo.y), dz = __fsub_rn(hi.z, lo.z);
    return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx)));
}

// ---------------------------------------------------------------- stage 1
__global__ void __launch_bounds__(kBB) k_tri_bounds(const float* __restrict__ pos, uint32_t nv,
                                                    const uint32_t* __restrict__ idx, uint32_t nt,
                                                    float4* __restrict__ tlo, float4* __restrict__ thi,
                                                    BuildStats* __restrict__ st) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t bl[3] = {kNone, kNone, kNone}, bh[3] = {0, 0, 0};
    uint32_t cl[3] = {kNone, kNone, kNone}, ch[3] = {0, 0, 0};
    uint32_t pm = 0;
    if (g < nt) {
        uint32_t v[3];
        bool bad = false;
        for (int j = 0; j < 3; ++j) {
            v[j] = idx[3 * (size_t)g + j];
            if (v[j] >= nv) {
                bad = true;
                v[j] = 0;
            }
        }
        if (bad) atomicOr(&st->bad_index, 1u);
        float lo[3], hi[3];
        for (int k = 0; k < 3; ++k) lo[k] = hi[k] = pos[3 * (size_t)v[0] + k];
        for (int j = 1; j < 3; ++j)
            for (int k = 0; k < 3; ++k) {
                float p = pos[3 * (size_t)v[j] + k];
                lo[k] = fminf(lo[k], p);
                hi[k] = fmaxf(hi[k], p);
            }
        tlo[g] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        thi[g] = make_float4(hi[0], hi[1], hi[2], 0.0f);
        float pmf = 0.0f;
        for (int k = 0; k < 3; ++k) {
            bl[k] = ord(lo[k]);
            bh[k] = ord(hi[k]);
            float c = __fmul_rn(0.5f, __fadd_rn(lo[k], hi[k]));
            cl[k] = ch[k] = ord(c);
            pmf = fmaxf(pmf, fmaxf(fabsf(lo[k]), fabsf(hi[k])));
        }
        pm = __float_as_uint(pmf);
    }
    for (int k = 0; k < 3; ++k) {
        bl[k] = __reduce_min_sync(0xffffffffu, bl[k]);
        bh[k] = __reduce_max_sync(0xffffffffu, bh[k]);
        cl[k] = __reduce_min_sync(0xffffffffu, cl[k]);
        ch[k] = __reduce_max_sync(0xffffffffu, ch[k]);
    }
    pm = __reduce_max_sync(0xffffffffu, pm);
    // Block reduction of the 13 values (one atomic per value and block:
    // per-warp atomics on the same 13 words serialised on 3M triangles).
    __shared__ uint32_t s_red[kBB / 32][13];
    const uint32_t warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            s_red[warp][k] = bl[k];
            s_red[warp][3 + k] = bh[k];
            s_red[warp][6 + k] = cl[k];
            s_red[warp][9 + k] = ch[k];
        }
        s_red[warp][12] = pm;
    }
    __syncthreads();
    if (threadIdx.x < 13) {
        const uint32_t q = threadIdx.x;
        const bool is_min = q < 3 || (q >= 6 && q < 9);
        uint32_t v = s_red[0][q];
        for (int w = 1; w < kBB / 32; ++w) v = is_min ? min(v, s_red[w][q]) : max(v, s_red[w][q]);
        uint32_t* dst = q < 3 ? &st->bmin[q] : q < 6 ? &st->bmax[q - 3] : q < 9 ? &st->cmin[q - 6]
                      : q < 12 ? &st->cmax[q - 9] : &st->pmax;
        if (is_min) atomicMin(dst, v);
        else atomicMax(dst, v);
    }
}

// ---------------------------------------------------------------- stage 2
__device__ __forceinline__ uint64_t spread21(uint32_t x) {
    uint64_t v = x & 0x1FFFFFu;
    v = (v | (v << 32)) & 0x1F00000000FFFFull;
    v = (v | (v << 16)) & 0x1F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

__global__ void __launch_bounds__(kBB) k_centroid_keys(const float4* __restrict__ tlo, const float4* __restrict__ thi,
                                                       uint32_t nt, const BuildStats* __restrict__ st,
                                                       uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nt) return;
    const float4 lo = tlo[g], hi = thi[g];
    const float c[3] = {__fmul_rn(0.5f, __fadd_rn(lo.x, hi.x)), __fmul_rn(0.5f, __fadd_rn(lo.y, hi.y)),
                        __fmul_rn(0.5f, __fadd_rn(lo.z, hi.z))};
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
        const float a = unord(st->cmin[k]), b = unord(st->cmax[k]);
        const float ext = __fsub_rn(b, a);
        float t = ext > 0.0f ? __fdiv_rn(__fsub_rn(c[k], a), ext) : 0.0f;
        t = fminf(fmaxf(t, 0.0f), 1.0f);
        q[k] = min((uint32_t)__fmul_rn(t, 2097151.0f), 2097151u);
    }
    keys[g] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[g] = g;
}

// Leaves in Morton order: node i is the triangle vals[i]; its record goes to
// slot i of the BVH2 triangle table.
__global__ void __launch_bounds__(kBB) k_leaves(const uint32_t* __restrict__ vals, uint32_t nt,
                                                const float4* __restrict__ tlo, const float4* __restrict__ thi,
                                                const float* __restrict__ pos, uint32_t nv,
                                                const uint32_t* __restrict__ idx,
                                                const uint32_t* __restrict__ geom_first, uint32_t ngeom,
                                                float4* __restrict__ nlo, float4* __restrict__ nhi,
                                                float4* __restrict__ recs, uint32_t* __restrict__ clusters) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const uint32_t g = vals[i];
    if (g >= nt) {
        raise_status(kErrBounds);
        return;
    }
    nlo[i] = tlo[g];
    nhi[i] = thi[g];
    // Geometry: the last entry of geom_first that is <= g (upper_bound - 1).
    uint32_t a = 0, b = ngeom;
    while (a < b) {
        uint32_t mid = (a + b) >> 1;
        if (geom_first[mid] <= g) a = mid + 1;
        else b = mid;
    }
    const uint32_t geom = a == 0 ? 0 : a - 1;
    const uint32_t prim = g - geom_first[geom];
    float4 r[3];
    for (int j = 0; j < 3; ++j) {
        uint32_t v = idx[3 * (size_t)g + j];
        if (v >= nv) v = 0;
        r[j] = make_float4(pos[3 * (size_t)v], pos[3 * (size_t)v + 1], pos[3 * (size_t)v + 2], 0.0f);
    }
    r[0].w = __int_as_float((int32_t)prim);
    r[1].w = __int_as_float((int32_t)geom);
    r[2].w = __uint_as_float(g);
    recs[3 * (size_t)i + 0] = r[0];
    recs[3 * (size_t)i + 1] = r[1];
    recs[3 * (size_t)i + 2] = r[2];
    clusters[i] = i;
}

// ----------------------------------------------------------- prefix sums
// Exclusive prefix sum of n u64 values in three launches: per-block sums,
// one block scanning those, per-block scan plus offset.
constexpr uint32_t kScanTile = kBB * kScanItems;

__device__ __forceinline__ uint64_t block_exclusive_u64(uint64_t v, uint64_t* s_warp, uint64_t* total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint64_t off = 0, sum = 0;
    for (int w = 0; w < kBB / 32; ++w) {
        uint64_t c = s_warp[w];
        if (w < (int)warp) off += c;
        sum += c;
    }
    __syncthreads();
    *total = sum;
    return off + x - v;
}

__global__ void __launch_bounds__(kBB) k_scan_reduce(const uint64_t* __restrict__ in, uint32_t n,
                                                     uint64_t* __restrict__ block_sums) {
    __shared__ uint64_t s_warp[kBB / 32];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint64_t s = 0;
    for (int j = 0; j < kScanItems; ++j)
        if (base + j < n) s += in[base + j];
    uint64_t total;
    block_exclusive_u64(s, s_warp, &total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kBB) k_scan_sums(uint64_t* __restrict__ block_sums, uint32_t nb,
                                                   uint64_t* __restrict__ grand_total) {
    __shared__ uint64_t s_warp[kBB / 32];
    uint64_t carry = 0;
    for (uint32_t c0 = 0; c0 < nb; c0 += kBB) {
        const uint32_t i = c0 + threadIdx.x;
        const uint64_t v = i < nb ? block_sums[i] : 0;
        uint64_t total;
        const uint64_t ex = block_exclusive_u64(v, s_warp, &total);
        if (i < nb) block_sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *grand_total = carry;
}

__global__ void __launch_bounds__(kBB) k_scan_apply(const uint64_t* __restrict__ in, uint32_t n,
                                                    const uint64_t* __restrict__ block_sums,
                                                    uint64_t* __restrict__ out) {
    __shared__ uint64_t s_warp[kBB / 32];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint64_t v[kScanItems], s = 0;
    for (int j = 0; j < kScanItems; ++j) {
        v[j] = base + j < n ? in[base + j] : 0;
        s += v[j];
    }
    uint64_t total;
    uint64_t run = block_exclusive_u64(s, s_warp, &total) + block_sums[blockIdx.x];
    for (int j = 0; j < kScanItems; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
}

struct Scan {
    uint64_t* block_sums = nullptr;  // >= ceil(n / kScanTile) entries
    uint64_t* total = nullptr;       // one entry
};

cudaError_t exclusive_scan(const uint64_t* in, uint64_t* out, uint32_t n, const Scan& sc, cudaStream_t s) {
    const uint32_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 0) return cudaMemsetAsync(sc.total, 0, sizeof(uint64_t), s);
    k_scan_reduce<<<nb, kBB, 0, s>>>(in, n, sc.block_sums);
    k_scan_sums<<<1, kBB, 0, s>>>(sc.block_sums, nb, sc.total);
    k_scan_apply<<<nb, kBB, 0, s>>>(in, n, sc.block_sums, out);
    count_launch();
    count_launch();
    count_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------- stage 3
// Nearest neighbour of every cluster within `radius` positions: the least
// merged surface area, ties to the smaller position.  For a fixed cluster
// that order is the order of (area, smaller position, larger position) over
// pairs, so the pair that is least in that order over all pairs is mutual
// and every iteration merges at least one pair.
__global__ void __launch_bounds__(kBB) k_ploc_nn(const uint32_t* __restrict__ cl, uint32_t m,
                                                 const float4* __restrict__ nlo, const float4* __restrict__ nhi,
                                                 uint32_t* __restrict__ nn, int radius) {
    __shared__ float4 s_lo[kBB + 2 * kPlocRMax], s_hi[kBB + 2 * kPlocRMax];
    const int R = radius < 1 ? 1 : (radius > kPlocRMax ? kPlocRMax : radius);
    const int b0 = (int)(blockIdx.x * kBB);
    for (int t = threadIdx.x; t < kBB + 2 * R; t += kBB) {
        const int j = b0 - R + t;
        if (j >= 0 && j < (int)m) {
            const uint32_t id = cl[j];
            s_lo[t] = nlo[id];
            s_hi[t] = nhi[id];
        }
    }
    __syncthreads();
    const int i = b0 + (int)threadIdx.x;
    if (i >= (int)m) return;
    const float4 alo = s_lo[threadIdx.x + R], ahi = s_hi[threadIdx.x + R];
    unsigned long long best = ~0ull;
    for (int d = -R; d <= R; ++d) {
        const int j = i + d;
        if (d == 0 || j < 0 || j >= (int)m) continue;
        const float4 blo = s_lo[threadIdx.x + R + d], bhi = s_hi[threadIdx.x + R + d];
        const float4 ulo = make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.0f);
        const float4 uhi = make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.0f);
        const unsigned long long key =
            ((unsigned long long)__float_as_uint(box_area(ulo, uhi)) << 32) | (uint32_t)j;
        best = key < best ? key : best;
    }
    nn[i] = (uint32_t)best;
}

// flags[i] = merge << 32 | keep: a mutual pair merges into its lower
// position; the upper one is dropped.
__global__ void __launch_bounds__(kBB) k_ploc_flags(const uint32_t* __restrict__ nn, uint32_t m,
                                                    uint64_t* __restrict__ flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t j = nn[i];
    const bool mutual = j < m && nn[j] == i;
    const bool merge = mutual && i < j;
    const bool keep = !(mutual && i > j);
    flags[i] = ((uint64_t)merge << 32) | (uint64_t)keep;
}

__global__ void __launch_bounds__(kBB) k_ploc_merge(const uint32_t* __restrict__ cl, const uint32_t* __restrict__ nn,
                                                    uint32_t m, const uint64_t* __restrict__ excl, uint32_t next_id,
                                                    uint32_t n_leaves, uint32_t cap, float4* __restrict__ nlo,
                                                    float4* __restrict__ nhi, int2* __restrict__ kids,
                                                    uint32_t* __restrict__ parent, uint32_t* __restrict__ cl_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t j = nn[i];
    const bool mutual = j < m && nn[j] == i;
    if (mutual && i > j) return;  // merged by its partner
    const uint64_t e = excl[i];
    const uint32_t posn = (uint32_t)e;
    if (!(mutual && i < j)) {
        cl_out[posn] = cl[i];
        return;
    }
    const uint32_t id = next_id + (uint32_t)(e >> 32);
    const uint32_t a = cl[i], b = cl[j];
    if (id >= cap || a >= cap || b >= cap || id < n_leaves) {
        raise_status(kErrBounds);
        return;
    }
    const float4 alo = nlo[a], ahi = nhi[a], blo = nlo[b], bhi = nhi[b];
    nlo[id] = make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.0f);
    nhi[id] = make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.0f);
    kids[id - n_leaves] = make_int2((int)a, (int)b);
    parent[a] = id;
    parent[b] = id;
    cl_out[posn] = id;
}

// ---------------------------------------------------------------- stage 4
// Inner node id (n_leaves .. 2 n_leaves - 2, in creation order) -> BVH2
// index 2 n_leaves - 2 - id: the root (created last) is node 0 and children
// come after their parents.
__global__ void __launch_bounds__(kBB) k_write_bvh2(uint32_t n, const int2* __restrict__ kids,
                                                    const float4* __restrict__ nlo, const float4* __restrict__ nhi,
                                                    const BuildStats* __restrict__ st, Bvh2Node* __restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k + 1 >= n) return;
    const uint32_t last = 2 * n - 2;
    const uint32_t index = last - (n + k);
    // Same growth as the host builder: delta = 2^-22 * P.
    const float delta = __fmul_rn(__uint_as_float(st->pmax), 0x1p-22f);
    Bvh2Node node;
    const int2 ch = kids[k];
    for (int c = 0; c < 2; ++c) {
        const uint32_t id = (uint32_t)(c == 0 ? ch.x : ch.y);
        const float4 lo = nlo[id], hi = nhi[id];
        const float lx = __fsub_rn(lo.x, delta), ly = __fsub_rn(lo.y, delta), lz = __fsub_rn(lo.z, delta);
        const float hx = __fadd_rn(hi.x, delta), hy = __fadd_rn(hi.y, delta), hz = __fadd_rn(hi.z, delta);
        const int o = c == 0 ? 0 : 4;
        node.f[o + 0] = lx;
        node.f[o + 1] = hx;
        node.f[o + 2] = ly;
        node.f[o + 3] = hy;
        node.f[8 + 2 * c] = lz;
        node.f[9 + 2 * c] = hz;
        node.link[c] = id < n ? (int32_t)~(id << 3) : (int32_t)(last - id);
    }
    node.link[2] = 0;
    node.link[3] = 0;
    out[index] = node;
}

// ---------------------------------------------------------------- stage 5
__device__ __forceinline__ float4 child_lo(const Bvh2Node& n, int c) {
    return c == 0 ? make_float4(n.f[0], n.f[2], n.f[8], 0.0f) : make_float4(n.f[4], n.f[6], n.f[10], 0.0f);
}
__device__ __forceinline__ float4 child_hi(const Bvh2Node& n, int c) {
    return c == 0 ? make_float4(n.f[1], n.f[3], n.f[9], 0.0f) : make_float4(n.f[5], n.f[7], n.f[11], 0.0f);
}

__device__ __forceinline__ Bvh2Node load_node(const Bvh2Node* nodes, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    Bvh2Node n;
    float4* q = reinterpret_cast<float4*>(&n);
    for (int k = 0; k < 4; ++k) q[k] = __ldg(p + k);
    return n;
}

// Bottom-up SAH collapse tables (the host's plan_sah): cost[i*8 + s-1] is
// the least cost of node i's subtree with at most s BVH8 children; how[i*8]
// -1 = one leaf child, 0 = one inner child; how[i*8 + s-1] (s > 1) 0 = same
// as s-1, a > 0 = a slots to child 0; split8[i] = child 0's slots when the
// node is a BVH8 inner node.
__global__ void __launch_bounds__(kBB) k_collapse_dp(uint32_t n, const Bvh2Node* __restrict__ nodes,
                                                     const uint32_t* __restrict__ parent,
                                                     uint32_t* __restrict__ visits, float* __restrict__ cost,
                                                     int8_t* __restrict__ how, int8_t* __restrict__ split8,
                                                     uint32_t* __restrict__ ntris, float tri_cost) {
    const uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= n) return;
    const uint32_t last = 2 * n - 2;
    uint32_t pid = parent[leaf];
    for (uint32_t guard = 0; pid != kNone && guard < n; ++guard) {
        if (pid < n || pid > last) {
            raise_status(kErrBounds);
            return;
        }
        const uint32_t i = last - pid;
        __threadfence();
        if (atomicAdd(&visits[i], 1u) == 0u) return;  // the sibling's thread computes it
        __threadfence();
        const Bvh2Node nd = load_node(nodes, i);
        float cc[2][8];
        uint32_t tc[2];
        float4 ulo, uhi;
        for (int c = 0; c < 2; ++c) {
            const float4 lo = child_lo(nd, c), hi = child_hi(nd, c);
            if (c == 0) {
                ulo = lo;
                uhi = hi;
            } else {
                ulo = make_float4(fminf(ulo.x, lo.x), fminf(ulo.y, lo.y), fminf(ulo.z, lo.z), 0.0f);
                uhi = make_float4(fmaxf(uhi.x, hi.x), fmaxf(uhi.y, hi.y), fmaxf(uhi.z, hi.z), 0.0f);
            }
            const int32_t link = nd.link[c];
            if (link < 0) {
                const uint32_t cnt = ((~(uint32_t)link) & 7u) + 1u;
                const float a = __fmul_rn(__fmul_rn(box_area(lo, hi), (float)cnt), tri_cost);
                for (int s = 0; s < 8; ++s) cc[c][s] = a;
                tc[c] = cnt;
            } else {
                for (int s = 0; s < 8; ++s) cc[c][s] = __ldcg(&cost[(size_t)link * 8 + s]);
                tc[c] = __ldcg(&ntris[link]);
            }
        }
        const float A = box_area(ulo, uhi);
        float dist[9];
        int8_t arg[9];
        for (int j = 2; j <= 8; ++j) {
            dist[j] = __int_as_float(0x7f800000);
            arg[j] = 1;
            for (int a = 1; a < j; ++a) {
                const float c = __fadd_rn(cc[0][a - 1], cc[1][j - a - 1]);
                if (c < dist[j]) {
                    dist[j] = c;
                    arg[j] = (int8_t)a;
                }
            }
        }
        const uint32_t t = tc[0] + tc[1];
        const float c_inner = __fadd_rn(A, dist[8]);
        const float c_leaf = t <= 3 ? __fmul_rn(__fmul_rn(A, (float)t), tri_cost) : __int_as_float(0x7f800000);
        float prev = fminf(c_leaf, c_inner);
        __stcg(&cost[(size_t)i * 8], prev);
        __stcg(&how[(size_t)i * 8], (int8_t)(c_leaf <= c_inner ? -1 : 0));
        for (int s = 2; s <= 8; ++s) {
            int8_t h = 0;
            if (dist[s] < prev) {
                prev = dist[s];
                h = arg[s];
            }
            __stcg(&cost[(size_t)i * 8 + s - 1], prev);
            __stcg(&how[(size_t)i * 8 + s - 1], h);
        }
        __stcg(&split8[i], arg[8]);
        __stcg(&ntris[i], t);
        pid = parent[pid];
    }
}

struct Child8 {
    int32_t link;      // BVH2 link
    uint32_t parent;   // BVH2 node holding the child's box
    uint8_t k;         // which child of `parent`
    uint8_t leaf;      // becomes a leaf child
    uint8_t tris;      // triangles of a leaf child
};

// The BVH8 children of BVH2 node `node` as an inner BVH8 node (the host's
// collect over split8): child 0's share first, each share depth-first.
__device__ int collect8(const Bvh2Node* __restrict__ nodes, const int8_t* __restrict__ how,
                        const int8_t* __restrict__ split8, const uint32_t* __restrict__ ntris, uint32_t node,
                        Child8* out) {
    struct Item {
        uint32_t p;
        uint8_t k, s;
    };
    Item st[16];
    int sp = 0, cnt = 0;
    const int a8 = split8[node];
    st[sp++] = {node, 1, (uint8_t)(8 - a8)};
    st[sp++] = {node, 0, (uint8_t)a8};
    while (sp > 0 && cnt < 8) {
        const Item it = st[--sp];
        const Bvh2Node pn = load_node(nodes, it.p);
        const int32_t link = pn.link[it.k];
        if (link < 0) {
            out[cnt++] = {link, it.p, it.k, 1, (uint8_t)(((~(uint32_t)link) & 7u) + 1u)};
            continue;
        }
        int s = it.s;
        while (s > 1 && how[(size_t)link * 8 + s - 1] == 0) --s;
        if (s <= 1) {
            const bool lf = how[(size_t)link * 8] == -1;
            out[cnt++] = {link, it.p, it.k, (uint8_t)(lf ? 1 : 0), (uint8_t)(lf ? ntris[link] : 0)};
            continue;
        }
        const int a = how[(size_t)link * 8 + s - 1];
        if (sp + 2 > 16) break;  // cannot happen: at most 8 children
        st[sp++] = {(uint32_t)link, 1, (uint8_t)(s - a)};
        st[sp++] = {(uint32_t)link, 0, (uint8_t)a};
    }
    return cnt;
}

__global__ void __launch_bounds__(kBB) k_emit_count(const uint2* __restrict__ tasks, uint32_t ntasks,
                                                    const Bvh2Node* __restrict__ nodes, const int8_t* __restrict__ how,
                                                    const int8_t* __restrict__ split8,
                                                    const uint32_t* __restrict__ ntris, uint64_t* __restrict__ counts) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    Child8 ch[8];
    const int nc = collect8(nodes, how, split8, ntris, tasks[t].y, ch);
    uint32_t inner = 0, tris = 0;
    for (int c = 0; c < nc; ++c) {
        if (ch[c].leaf) tris += ch[c].tris;
        else ++inner;
    }
    counts[t] = ((uint64_t)inner << 32) | tris;
}

// Triangles of a leaf child (a subtree of at most three triangles), depth
// first, child 0 first, like the host's gather_tris.
__device__ int gather3(const Bvh2Node* __restrict__ nodes, int32_t link, uint32_t* recs) {
    int32_t st[8];
    int sp = 0, cnt = 0;
    st[sp++] = link;
    while (sp > 0) {
        const int32_t l = st[--sp];
        if (l < 0) {
            const uint32_t code = ~(uint32_t)l;
            const uint32_t first = code >> 3, c = (code & 7u) + 1u;
            for (uint32_t q = 0; q < c && cnt < 3; ++q) recs[cnt++] = first + q;
            continue;
        }
        const Bvh2Node nd = load_node(nodes, (uint32_t)l);
        if (sp + 2 > 8) break;
        st[sp++] = nd.link[1];
        st[sp++] = nd.link[0];
    }
    return cnt;
}

__global__ void __launch_bounds__(kBB) k_emit_write(const uint2* __restrict__ tasks, uint32_t ntasks,
                                                    const uint64_t* __restrict__ excl, uint32_t node_base,
                                                    uint32_t tri_base0, uint32_t node_cap, uint32_t tri_cap,
                                                    const Bvh2Node* __restrict__ nodes,
                                                    const int8_t* __restrict__ how, const int8_t* __restrict__ split8,
                                                    const uint32_t* __restrict__ ntris,
                                                    const float4* __restrict__ recs2, Bvh8Node* __restrict__ out,
                                                    float4* __restrict__ recs8,
                                                    uint2* __restrict__ next_tasks) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    const uint2 task = tasks[t];
    Child8 ch[8];
    const int nc = collect8(nodes, how, split8, ntris, task.y, ch);
    const uint64_t e = excl[t];
    const uint32_t inner_off = (uint32_t)(e >> 32), tri_off0 = (uint32_t)e;
    Bvh8Node node;
    memset(&node, 0, sizeof(node));
    float4 clo[8], chi[8];
    float nlo[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
    float nhi[3] = {-nlo[0], -nlo[1], -nlo[2]};
    for (int c = 0; c < nc; ++c) {
        const Bvh2Node pn = load_node(nodes, ch[c].parent);
        clo[c] = child_lo(pn, ch[c].k);
        chi[c] = child_hi(pn, ch[c].k);
        nlo[0] = fminf(nlo[0], clo[c].x);
        nlo[1] = fminf(nlo[1], clo[c].y);
        nlo[2] = fminf(nlo[2], clo[c].z);
        nhi[0] = fmaxf(nhi[0], chi[c].x);
        nhi[1] = fmaxf(nhi[1], chi[c].y);
        nhi[2] = fmaxf(nhi[2], chi[c].z);
    }
    // Quantisation grid (the host's emit_children): the smallest power-of-two
    // scale whose 255 steps from the box minimum reach the box maximum.
    float scale[3];
    for (int k = 0; k < 3; ++k) {
        node.p[k] = nlo[k];
        const float ext = __fsub_rn(nhi[k], nlo[k]);
        int ex = -126;
        if (ext > 0.0f) {
            int e2;
            frexpf(__fdiv_rn(ext, 255.0f), &e2);
            ex = e2;
        }
        for (int guard = 0; guard < 300; ++guard) {
            ex = max(-126, min(127, ex));
            scale[k] = ldexpf(1.0f, ex);
            const float top = __fadd_rn(node.p[k], __fmul_rn(255.0f, scale[k]));
            if (top >= nhi[k] || ex == 127) break;
            ++ex;
        }
        node.e[k] = (uint8_t)(ex + 127);
    }
    // Slots: greedy by descending octant score, ties to the lower (child,
    // slot) pair, as the host's stable sort.
    float pc[3];
    for (int k = 0; k < 3; ++k) pc[k] = __fmul_rn(0.5f, __fadd_rn(nlo[k], nhi[k]));
    float off[8][3];
    for (int c = 0; c < nc; ++c) {
        off[c][0] = __fsub_rn(__fmul_rn(0.5f, __fadd_rn(clo[c].x, chi[c].x)), pc[0]);
        off[c][1] = __fsub_rn(__fmul_rn(0.5f, __fadd_rn(clo[c].y, chi[c].y)), pc[1]);
        off[c][2] = __fsub_rn(__fmul_rn(0.5f, __fadd_rn(clo[c].z, chi[c].z)), pc[2]);
    }
    int slot_of[8], child_at[8];
    for (int q = 0; q < 8; ++q) slot_of[q] = child_at[q] = -1;
    for (int round = 0; round < nc; ++round) {
        float best = 0.0f;
        int bc = -1, bs = -1;
        for (int c = 0; c < nc; ++c) {
            if (slot_of[c] >= 0) continue;
            for (int sl = 0; sl < 8; ++sl) {
                if (child_at[sl] >= 0) continue;
                float sc = 0.0f;
                for (int k = 0; k < 3; ++k) sc = __fadd_rn(sc, ((sl >> k) & 1) ? -off[c][k] : off[c][k]);
                if (bc < 0 || sc > best) {
                    best = sc;
                    bc = c;
                    bs = sl;
                }
            }
        }
        if (bc < 0) break;
        slot_of[bc] = bs;
        child_at[bs] = bc;
    }
    const uint32_t child_base = node_base + inner_off;
    const uint32_t tri_base = tri_base0 + tri_off0;
    node.child_base = child_base;
    node.tri_base = tri_base;
    uint32_t inner_i = 0, tri_off = 0;
    for (int sl = 0; sl < 8; ++sl) {
        const int ci = child_at[sl];
        if (ci < 0) continue;
        const Child8& c = ch[ci];
        const float lo3[3] = {clo[ci].x, clo[ci].y, clo[ci].z}, hi3[3] = {chi[ci].x, chi[ci].y, chi[ci].z};
        for (int k = 0; k < 3; ++k) {
            const float sc = scale[k];
            const float lo = floorf(__fdiv_rn(__fsub_rn(lo3[k], node.p[k]), sc));
            const float hi = ceilf(__fdiv_rn(__fsub_rn(hi3[k], node.p[k]), sc));
            int ql = (int)fmaxf(0.0f, fminf(255.0f, lo));
            int qh = (int)fmaxf(0.0f, fminf(255.0f, hi));
            while (ql > 0 && __fadd_rn(node.p[k], __fmul_rn((float)ql, sc)) > lo3[k]) --ql;
            while (qh < 255 && __fadd_rn(node.p[k], __fmul_rn((float)qh, sc)) < hi3[k]) ++qh;
            uint8_t* qlo = k == 0 ? node.qlo_x : (k == 1 ? node.qlo_y : node.qlo_z);
            uint8_t* qhi = k == 0 ? node.qhi_x : (k == 1 ? node.qhi_y : node.qhi_z);
            qlo[sl] = (uint8_t)ql;
            qhi[sl] = (uint8_t)qh;
        }
        if (c.leaf) {
            uint32_t r[3];
            const int cnt = gather3(nodes, c.link, r);
            const uint32_t unary = cnt == 1 ? 1u : (cnt == 2 ? 3u : 7u);
            node.meta[sl] = (uint8_t)((unary << 5) | tri_off);
            for (int q = 0; q < cnt; ++q) {
                const uint32_t dst = tri_base + tri_off + q;
                if (dst >= tri_cap) {
                    raise_status(kErrBounds);
                    continue;
                }
                const float4 a = recs2[3 * (size_t)r[q]], b = recs2[3 * (size_t)r[q] + 1],
                             cc = recs2[3 * (size_t)r[q] + 2];
                recs8[3 * (size_t)dst] = a;
                recs8[3 * (size_t)dst + 1] = b;
                recs8[3 * (size_t)dst + 2] = cc;
            }
            tri_off += (uint32_t)cnt;
        } else {
            node.imask |= (uint8_t)(1u << sl);
            node.meta[sl] = (uint8_t)((1u << 5) | (24u + (uint32_t)sl));
            if (child_base + inner_i < node_cap) next_tasks[inner_off + inner_i] = make_uint2(child_base + inner_i, (uint32_t)c.link);
            else raise_status(kErrBounds);
            ++inner_i;
        }
    }
    if (task.x < node_cap) out[task.x] = node;
    else raise_status(kErrBounds);
}

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    return dev_malloc(reinterpret_cast<void**>(p), std::max<size_t>(1, count) * sizeof(T));
}

unsigned blocks(uint64_t n) { return (unsigned)((n + kBB - 1) / kBB); }

}  // namespace

cudaError_t build_scene_device(const float* positions_dev, uint32_t num_vertices, const uint32_t* indices_dev,
                               uint32_t num_triangles, const uint32_t* geom_first_dev, uint32_t num_geoms,
                               bool want8, cudaStream_t s, DeviceBuild* out) {
    const uint32_t n = num_triangles;
    if (n < 2 || !out || num_geoms == 0) return cudaErrorInvalidValue;
    *out = DeviceBuild{};
    cudaError_t e = cudaSuccess;
    // Temporaries, freed at the end.
    float4 *tlo = nullptr, *thi = nullptr, *nlo = nullptr, *nhi = nullptr;
    uint64_t *keys = nullptr, *flags = nullptr, *excl = nullptr, *bsums = nullptr, *total = nullptr;
    uint32_t *vals = nullptr, *cl = nullptr, *cl2 = nullptr, *nn = nullptr, *parent = nullptr;
    int2* kids = nullptr;
    BuildStats* st = nullptr;
    unsigned char* sort_scratch = nullptr;
    float* cost = nullptr;
    int8_t *how = nullptr, *split8 = nullptr;
    uint32_t *ntris = nullptr, *visits = nullptr;
    uint2 *tasks = nullptr, *tasks2 = nullptr;
    Bvh8Node* nodes8_tmp = nullptr;
    Bvh2Node* nodes2 = nullptr;
    float4* recs2 = nullptr;
    float4* recs8 = nullptr;
    Bvh8Node* nodes8 = nullptr;
    const size_t ninner = (size_t)n - 1, nall = 2 * (size_t)n - 1;
    const size_t sort_bytes = sort_scratch_bytes(n, 63);
    const uint32_t nb = (n + kScanTile - 1) / kScanTile;
    Scan scan;
    uint64_t host_total = 0;
    uint32_t m = n, next_id = n, iterations = 0;

#define WFPT_TRY(x)                      \
    do {                                 \
        if ((e = (x)) != cudaSuccess) goto done; \
    } while (0)

    WFPT_TRY(dalloc(&tlo, n));
    WFPT_TRY(dalloc(&thi, n));
    WFPT_TRY(dalloc(&nlo, nall));
    WFPT_TRY(dalloc(&nhi, nall));
    WFPT_TRY(dalloc(&keys, n));
    WFPT_TRY(dalloc(&vals, n));
    WFPT_TRY(dalloc(&flags, n));
    WFPT_TRY(dalloc(&excl, n));
    WFPT_TRY(dalloc(&bsums, nb + 1));
    WFPT_TRY(dalloc(&total, 1));
    WFPT_TRY(dalloc(&cl, n));
    WFPT_TRY(dalloc(&cl2, n));
    WFPT_TRY(dalloc(&nn, n));
    WFPT_TRY(dalloc(&parent, nall));
    WFPT_TRY(dalloc(&kids, ninner));
    WFPT_TRY(dalloc(&st, 1));
    WFPT_TRY(dalloc(&sort_scratch, sort_bytes));
    WFPT_TRY(dalloc(&nodes2, ninner));
    WFPT_TRY(dalloc(&recs2, 3 * (size_t)n));
    scan.block_sums = bsums;
    scan.total = total;

    {  // stage 1: bounds
        BuildStats init;
        for (int k = 0; k < 3; ++k) {
            init.bmin[k] = init.cmin[k] = kNone;
            init.bmax[k] = init.cmax[k] = 0;
        }
        init.pmax = 0;
        init.bad_index = 0;
        WFPT_TRY(cudaMemcpyAsync(st, &init, sizeof(init), cudaMemcpyHostToDevice, s));
        k_tri_bounds<<<blocks(n), kBB, 0, s>>>(positions_dev, num_vertices, indices_dev, n, tlo, thi, st);
        count_launch();
        WFPT_TRY(cudaGetLastError());
        BuildStats got;
        WFPT_TRY(cudaMemcpyAsync(&got, st, sizeof(got), cudaMemcpyDeviceToHost, s));
        WFPT_TRY(cudaStreamSynchronize(s));
        if (got.bad_index) {
            e = cudaErrorInvalidValue;
            goto done;
        }
        for (int k = 0; k < 3; ++k) {
            const uint32_t lo = (got.bmin[k] & 0x80000000u) ? (got.bmin[k] & 0x7FFFFFFFu) : ~got.bmin[k];
            const uint32_t hi = (got.bmax[k] & 0x80000000u) ? (got.bmax[k] & 0x7FFFFFFFu) : ~got.bmax[k];
            std::memcpy(&out->bounds_min[k], &lo, 4);
            std::memcpy(&out->bounds_max[k], &hi, 4);
        }
    }
    // stage 2: keys, sort, leaves
    k_centroid_keys<<<blocks(n), kBB, 0, s>>>(tlo, thi, n, st, keys, vals);
    count_launch();
    WFPT_TRY(cudaGetLastError());
    WFPT_TRY(launch_sort_pairs(keys, vals, n, nullptr, 63, sort_scratch, sort_bytes, s));
    k_leaves<<<blocks(n), kBB, 0, s>>>(vals, n, tlo, thi, positions_dev, num_vertices, indices_dev, geom_first_dev,
                                       num_geoms, nlo, nhi, recs2, cl);
    count_launch();
    WFPT_TRY(cudaGetLastError());
    WFPT_TRY(cudaMemsetAsync(parent, 0xFF, nall * sizeof(uint32_t), s));
    // stage 3: PLOC until one cluster is left (each pass merges at least one
    // pair, so n passes bound the loop).
    while (m > 1) {
        if (++iterations > n) {
            e = cudaErrorUnknown;
            goto done;
        }
        k_ploc_nn<<<blocks(m), kBB, 0, s>>>(cl, m, nlo, nhi, nn, g_ploc_radius);
        k_ploc_flags<<<blocks(m), kBB, 0, s>>>(nn, m, flags);
        count_launch();
        count_launch();
        WFPT_TRY(cudaGetLastError());
        WFPT_TRY(exclusive_scan(flags, excl, m, scan, s));
        k_ploc_merge<<<blocks(m), kBB, 0, s>>>(cl, nn, m, excl, next_id, n, (uint32_t)nall, nlo, nhi, kids, parent,
                                               cl2);
        count_launch();
        WFPT_TRY(cudaGetLastError());
        WFPT_TRY(cudaMemcpyAsync(&host_total, total, sizeof(host_total), cudaMemcpyDeviceToHost, s));
        WFPT_TRY(cudaStreamSynchronize(s));
        const uint32_t merges = (uint32_t)(host_total >> 32), kept = (uint32_t)host_total;
        if (merges == 0 || kept >= m) {
            e = cudaErrorUnknown;  // no progress: cannot happen (see k_ploc_nn)
            goto done;
        }
        next_id += merges;
        m = kept;
        std::swap(cl, cl2);
    }
    if (next_id != nall) {
        e = cudaErrorUnknown;
        goto done;
    }
    out->ploc_iterations = iterations;
    // stage 4: BVH2 in the traversal format
    k_write_bvh2<<<blocks(ninner), kBB, 0, s>>>(n, kids, nlo, nhi, st, nodes2);
    count_launch();
    WFPT_TRY(cudaGetLastError());
    // stage 5: BVH8
    if (want8) {
        WFPT_TRY(dalloc(&cost, 8 * ninner));
        WFPT_TRY(dalloc(&how, 8 * ninner));
        WFPT_TRY(dalloc(&split8, ninner));
        WFPT_TRY(dalloc(&ntris, ninner));
        WFPT_TRY(dalloc(&visits, ninner));
        WFPT_TRY(dalloc(&tasks, ninner));
        WFPT_TRY(dalloc(&tasks2, ninner));
        WFPT_TRY(dalloc(&nodes8_tmp, ninner));
        WFPT_TRY(dalloc(&recs8, 3 * (size_t)n));
        WFPT_TRY(cudaMemsetAsync(visits, 0, ninner * sizeof(uint32_t), s));
        k_collapse_dp<<<blocks(n), kBB, 0, s>>>(n, nodes2, parent, visits, cost, how, split8, ntris,
                                                (float)get_bvh8_tri_cost_pct() * 0.01f);
        count_launch();
        WFPT_TRY(cudaGetLastError());
        uint2 root = make_uint2(0u, 0u);
        WFPT_TRY(cudaMemcpyAsync(tasks, &root, sizeof(root), cudaMemcpyHostToDevice, s));
        uint32_t ntasks = 1, node_count = 1, tri_count = 0;
        for (int level = 0; ntasks > 0; ++level) {
            if (level > 64 || ntasks > ninner) {
                e = cudaErrorUnknown;
                goto done;
            }
            k_emit_count<<<blocks(ntasks), kBB, 0, s>>>(tasks, ntasks, nodes2, how, split8, ntris, flags);
            count_launch();
            WFPT_TRY(cudaGetLastError());
            WFPT_TRY(exclusive_scan(flags, excl, ntasks, scan, s));
            k_emit_write<<<blocks(ntasks), kBB, 0, s>>>(tasks, ntasks, excl, node_count, tri_count,
                                                        (uint32_t)ninner, n, nodes2, how, split8, ntris, recs2,
                                                        nodes8_tmp, recs8, tasks2);
            count_launch();
            WFPT_TRY(cudaGetLastError());
            WFPT_TRY(cudaMemcpyAsync(&host_total, total, sizeof(host_total), cudaMemcpyDeviceToHost, s));
            WFPT_TRY(cudaStreamSynchronize(s));
            const uint32_t inner = (uint32_t)(host_total >> 32), tris = (uint32_t)host_total;
            node_count += inner;
            tri_count += tris;
            ntasks = inner;
            std::swap(tasks, tasks2);
            if (node_count > ninner || tri_count > n) {
                e = cudaErrorUnknown;
                goto done;
            }
        }
        if (tri_count != n) {
            e = cudaErrorUnknown;
            goto done;
        }
        WFPT_TRY(dalloc(&nodes8, node_count));
        WFPT_TRY(cudaMemcpyAsync(nodes8, nodes8_tmp, node_count * sizeof(Bvh8Node), cudaMemcpyDeviceToDevice, s));
        out->bvh8_count = node_count;
    }
    WFPT_TRY(cudaStreamSynchronize(s));
    {
        uint32_t flags_h = 0;
        WFPT_TRY(status_build(&flags_h));
        if (flags_h) {
            e = cudaErrorUnknown;
            goto done;
        }
    }
    out->bvh2_nodes = nodes2;
    out->bvh2_tris = recs2;
    out->bvh2_count = (uint32_t)ninner;
    out->bvh8_nodes = nodes8;
    out->bvh8_tris = recs8;
    nodes2 = nullptr;
    recs2 = nullptr;
    nodes8 = nullptr;
    recs8 = nullptr;
#undef WFPT_TRY
done:
    for (void* p : {(void*)tlo, (void*)thi, (void*)nlo, (void*)nhi, (void*)keys, (void*)flags, (void*)excl,
                    (void*)bsums, (void*)total, (void*)vals, (void*)cl, (void*)cl2, (void*)nn, (void*)parent,
                    (void*)kids, (void*)st, (void*)sort_scratch, (void*)cost, (void*)how, (void*)split8,
                    (void*)ntris, (void*)visits, (void*)tasks, (void*)tasks2, (void*)nodes8_tmp, (void*)nodes2,
                    (void*)recs2, (void*)recs8, (void*)nodes8})
        if (p) cudaFree(p);
    return e;
}

}  // namespace wfpt
