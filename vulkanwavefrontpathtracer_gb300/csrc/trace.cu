// Software BVH traversal: replaces trace.comp's rayQuery (trace.comp:50-84)
// on a GPU without RT cores.
//
// Plain form  (WFPT_BVH2_FP32): binary BVH, each 64-byte node holds both
//   children's FP32 boxes; one thread per ray, while-while traversal with a
//   per-thread stack.
// Chosen form (WFPT_BVH8_Q8):   8-wide BVH, 80-byte nodes with an FP32
//   origin, per-axis power-of-two scales and 8-bit child boxes rounded
//   outward; children visited in ray-octant order, node groups on the stack
//   (Ylitie, Karras, Laine: "Efficient Incoherent Ray Traversal on GPUs
//   Through Compressed Wide BVHs", HPG 2017).  Persistent warps: a lane
//   whose ray is done takes the next ray from a global counter (one atomic
//   per warp for all idle lanes), so warps stay full on incoherent rays.
// Both use the watertight ray/triangle test of Woop, Benthin and Wald
// (JCGT 2013), evaluated without FMA contraction, and the same closest-hit
// rule (smallest t, ties to the smaller global triangle index), so both
// forms return identical hits.
#include <atomic>

#include "common.cuh"
#include "scene.h"
#include "stages.cuh"
#include "trace.cuh"

namespace wfpt {

cudaError_t status_trace(uint32_t* out) { return read_and_clear_status(out); }

constexpr int kStack2 = 64;
constexpr int kStack8 = 32;
// Relative slack on box exit distances (about 2*gamma(3) for FP32).
constexpr float kBoxSlack = 1.0000004f;
constexpr uint32_t kNoRay = 0xFFFFFFFFu;

// Work counters of the counting kernel variants: node visits, triangle
// tests, rays, warp loop iterations (persistent kernel only).
static __device__ unsigned long long g_counts[4];

__device__ __forceinline__ void add_counts(uint32_t nodes, uint32_t tris, uint32_t rays, uint32_t iters) {
    atomicAdd(&g_counts[0], (unsigned long long)nodes);
    atomicAdd(&g_counts[1], (unsigned long long)tris);
    atomicAdd(&g_counts[2], (unsigned long long)rays);
    if (iters) atomicAdd(&g_counts[3], (unsigned long long)iters);
}

struct RayT {
    f3 o;
    f3 inv;
    f3 oinv;  // o * inv
    float tmin;
    int kx, ky, kz;
    float sx, sy, sz;
    uint32_t oct;  // bit k = sign bit of d[k]
};

__device__ __forceinline__ float comp(const f3& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ float safe_inv(float d) {
    const float eps = 1e-20f;
    float a = fabsf(d) > eps ? d : copysignf(eps, d);
    return __fdiv_rn(1.0f, a);
}

__device__ __forceinline__ RayT setup_ray(const float4& r0, const float4& r1) {
    RayT r;
    r.o = mk(r0.x, r0.y, r0.z);
    f3 d = mk(r1.x, r1.y, r1.z);
    r.tmin = r0.w;
    r.inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    r.oinv = mul(r.o, r.inv);
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (comp(d, kz) < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    float dz = comp(d, kz);
    r.sx = __fdiv_rn(comp(d, kx), dz);
    r.sy = __fdiv_rn(comp(d, ky), dz);
    r.sz = __fdiv_rn(1.0f, dz);
    // Sign bits (not d < 0): -0.0 has a negative reciprocal in safe_inv, and
    // the BVH8 near/far plane choice must agree with the sign of inv.
    r.oct = (__float_as_uint(d.x) >> 31) | ((__float_as_uint(d.y) >> 31) << 1) |
            ((__float_as_uint(d.z) >> 31) << 2);
    return r;
}

// Closest-hit state: distance, tie-break key (global triangle index) and
// the triangle record index; barycentrics are recomputed once at the end.
struct HitS {
    float t;
    uint32_t key;
    uint32_t rec;
};

struct Uvw {
    float U, V, W, det, T;
    bool edge_ok;
};

// Woop-Benthin-Wald edge functions and scaled distance for one triangle,
// from the ray origin, its axis permutation and shear constants.
__device__ __forceinline__ Uvw tri_uvw(const f3& org, int kx, int ky, int kz, float sx, float sy, float sz,
                                       const float4& a4, const float4& b4, const float4& c4) {
    f3 A = sub(mk(a4.x, a4.y, a4.z), org);
    f3 B = sub(mk(b4.x, b4.y, b4.z), org);
    f3 C = sub(mk(c4.x, c4.y, c4.z), org);
    float Akz = comp(A, kz), Bkz = comp(B, kz), Ckz = comp(C, kz);
    float Ax = __fsub_rn(comp(A, kx), __fmul_rn(sx, Akz));
    float Ay = __fsub_rn(comp(A, ky), __fmul_rn(sy, Akz));
    float Bx = __fsub_rn(comp(B, kx), __fmul_rn(sx, Bkz));
    float By = __fsub_rn(comp(B, ky), __fmul_rn(sy, Bkz));
    float Cx = __fsub_rn(comp(C, kx), __fmul_rn(sx, Ckz));
    float Cy = __fsub_rn(comp(C, ky), __fmul_rn(sy, Ckz));
    Uvw q;
    q.U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    q.V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    q.W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (q.U == 0.0f || q.V == 0.0f || q.W == 0.0f) {
        double cxby = (double)Cx * (double)By, cybx = (double)Cy * (double)Bx;
        q.U = (float)(cxby - cybx);
        double axcy = (double)Ax * (double)Cy, aycx = (double)Ay * (double)Cx;
        q.V = (float)(axcy - aycx);
        double bxay = (double)Bx * (double)Ay, byax = (double)By * (double)Ax;
        q.W = (float)(bxay - byax);
    }
    q.edge_ok = !((q.U < 0.0f || q.V < 0.0f || q.W < 0.0f) && (q.U > 0.0f || q.V > 0.0f || q.W > 0.0f));
    q.det = __fadd_rn(__fadd_rn(q.U, q.V), q.W);
    float Az = __fmul_rn(sz, Akz), Bz = __fmul_rn(sz, Bkz), Cz = __fmul_rn(sz, Ckz);
    q.T = __fadd_rn(__fadd_rn(__fmul_rn(q.U, Az), __fmul_rn(q.V, Bz)), __fmul_rn(q.W, Cz));
    return q;
}

__device__ __forceinline__ Uvw tri_uvw(const RayT& r, const float4& a4, const float4& b4, const float4& c4) {
    return tri_uvw(r.o, r.kx, r.ky, r.kz, r.sx, r.sy, r.sz, a4, b4, c4);
}

// Watertight test of record `rec`; on acceptance updates `h`.
__device__ __forceinline__ bool intersect_tri(const RayT& r, const float4* __restrict__ tris, uint32_t rec,
                                              HitS& h) {
    float4 a4 = __ldg(&tris[3 * rec + 0]);
    float4 b4 = __ldg(&tris[3 * rec + 1]);
    float4 c4 = __ldg(&tris[3 * rec + 2]);
    Uvw q = tri_uvw(r, a4, b4, c4);
    if (!q.edge_ok || q.det == 0.0f) return false;
    float t = __fdiv_rn(q.T, q.det);
    if (!(t >= r.tmin)) return false;
    uint32_t key = __float_as_uint(c4.w);
    if (!(t < h.t || (t == h.t && key < h.key))) return false;
    h.t = t;
    h.key = key;
    h.rec = rec;
    return true;
}

// Writes the RayResult of a finished ray (trace.comp:66-84).
__device__ __forceinline__ void write_hit(int4* __restrict__ results, uint32_t ri, const RayT& r,
                                          const float4* __restrict__ tris, const HitS& h, bool found) {
    int4 out;
    if (found) {
        float4 a4 = __ldg(&tris[3 * h.rec + 0]);
        float4 b4 = __ldg(&tris[3 * h.rec + 1]);
        float4 c4 = __ldg(&tris[3 * h.rec + 2]);
        Uvw q = tri_uvw(r, a4, b4, c4);  // same inputs, same edge functions as at acceptance
        float u = __fdiv_rn(q.V, q.det), v = __fdiv_rn(q.W, q.det);
        out = make_int4(__float_as_int(a4.w), __float_as_int(b4.w), __float_as_int(h.t), (int)pack_unorm2x16(u, v));
    } else {
        out = make_int4(-1, -1, __float_as_int(-1.0f), 0);
    }
    results[ri] = out;
}

__device__ __forceinline__ void write_miss(int4* __restrict__ results, uint32_t ri) {
    results[ri] = make_int4(-1, -1, __float_as_int(-1.0f), 0);
}

// ------------------------------------------------------------ BVH2 (plain)
__device__ __forceinline__ void box2(const RayT& r, float lox, float hix, float loy, float hiy, float loz,
                                     float hiz, float tcur, float& tnear, bool& hit) {
    float x0 = __fmaf_rn(lox, r.inv.x, -r.oinv.x), x1 = __fmaf_rn(hix, r.inv.x, -r.oinv.x);
    float y0 = __fmaf_rn(loy, r.inv.y, -r.oinv.y), y1 = __fmaf_rn(hiy, r.inv.y, -r.oinv.y);
    float z0 = __fmaf_rn(loz, r.inv.z, -r.oinv.z), z1 = __fmaf_rn(hiz, r.inv.z, -r.oinv.z);
    float tn = fmaxf(max3f(fminf(x0, x1), fminf(y0, y1), fminf(z0, z1)), r.tmin);
    float tf = fminf(min3f(fmaxf(x0, x1), fmaxf(y0, y1), fmaxf(z0, z1)), tcur);
    tnear = tn;
    hit = tn <= tf * kBoxSlack;
}

template <bool CLOSEST, bool COUNT>
__global__ void __launch_bounds__(kBlock) k_trace_bvh2(const float4* __restrict__ nodes,
                                                       const float4* __restrict__ tris,
                                                       const float4* __restrict__ rays, int4* __restrict__ results,
                                                       const uint32_t* __restrict__ ray_index, uint32_t n,
                                                       const uint32_t* __restrict__ n_dev) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= load_count(n, n_dev)) return;
    uint32_t ri = ray_index ? ray_index[i] : i;
    float4 r0 = rays[2 * ri + 0];
    float4 r1 = rays[2 * ri + 1];
    if (!(r1.w >= r0.w)) {  // tmax < tmin (or NaN): empty interval
        write_miss(results, ri);
        return;
    }
    RayT r = setup_ray(r0, r1);
    HitS h{r1.w, 0xFFFFFFFFu, 0u};
    bool found = false;
    uint32_t c_nodes = 0, c_tris = 0;
    int stack[kStack2];
    int sp = 0;
    int node = 0;
    bool done = false;
    while (!done) {
        // Inner nodes.
        while (node >= 0) {
            if (COUNT) ++c_nodes;
            float4 a = __ldg(&nodes[4 * node + 0]);
            float4 b = __ldg(&nodes[4 * node + 1]);
            float4 c = __ldg(&nodes[4 * node + 2]);
            int4 l = __ldg(reinterpret_cast<const int4*>(&nodes[4 * node + 3]));
            float t0, t1;
            bool h0, h1;
            box2(r, a.x, a.y, a.z, a.w, c.x, c.y, h.t, t0, h0);
            box2(r, b.x, b.y, b.z, b.w, c.z, c.w, h.t, t1, h1);
            if (h0 && h1) {
                int nearc = l.x, farc = l.y;
                if (t1 < t0) {
                    nearc = l.y;
                    farc = l.x;
                }
                if (sp < kStack2) {
                    stack[sp++] = farc;
                } else {
                    raise_status(kErrBounds);
                }
                node = nearc;
            } else if (h0) {
                node = l.x;
            } else if (h1) {
                node = l.y;
            } else {
                if (sp == 0) {
                    done = true;
                    break;
                }
                node = stack[--sp];
            }
        }
        if (done) break;
        // Leaves.
        while (node < 0) {
            uint32_t code = ~(uint32_t)node;
            uint32_t first = code >> 3, cnt = (code & 7u) + 1u;
            for (uint32_t k = 0; k < cnt; ++k) {
                if (COUNT) ++c_tris;
                if (intersect_tri(r, tris, first + k, h)) {
                    found = true;
                    if (!CLOSEST) break;
                }
            }
            if (!CLOSEST && found) {
                done = true;
                break;
            }
            if (sp == 0) {
                done = true;
                break;
            }
            node = stack[--sp];
        }
    }
    write_hit(results, ri, r, tris, h, found);
    if (COUNT) add_counts(c_nodes, c_tris, 1u, 0u);
}

// --------------------------------------------------------- BVH8 (chosen)
__device__ __forceinline__ uint32_t byte_of(uint32_t w, int b) { return (w >> (8 * b)) & 0xFFu; }

// Byte b of w as the exact float 2^15 + q: one PRMT places the byte in
// mantissa bits 8..15 of 2^15 (bits 0x4700qq00).  The 2^15 bias is folded
// into the node's slab offsets (intersect_node8), so a plane costs one PRMT
// and one FMA.
__device__ __forceinline__ float q2f(uint32_t w, int b) {
    return __uint_as_float(__byte_perm(w, 0x47000000u, 0x7604u | ((uint32_t)b << 4)));
}

// Intersects the eight children of a BVH8 node.  Returns the hit mask:
// bits 24..31 inner children (octant-permuted slot order, highest first),
// bits 0..23 triangles relative to *tri_base; *child_base and *imask out.
__device__ __forceinline__ uint32_t intersect_node8(const float4* __restrict__ nd, const RayT& r, float tcur,
                                                    uint32_t& child_base, uint32_t& tri_base, uint32_t& imask) {
    float4 n0 = __ldg(nd + 0);
    float4 n1 = __ldg(nd + 1);
    float4 n2 = __ldg(nd + 2);
    float4 n3 = __ldg(nd + 3);
    float4 n4 = __ldg(nd + 4);
    const uint32_t oct = r.oct;
    uint32_t ew = __float_as_uint(n0.w);
    float scx = __uint_as_float((ew & 0xFFu) << 23);
    float scy = __uint_as_float(((ew >> 8) & 0xFFu) << 23);
    float scz = __uint_as_float(((ew >> 16) & 0xFFu) << 23);
    imask = ew >> 24;
    child_base = __float_as_uint(n1.x);
    tri_base = __float_as_uint(n1.y);
    // Slab distance = q * (scale*inv) + (p - o) * inv, evaluated as
    // (2^15 + q) * a + (b - 2^15 a).  The folded offset is rounded twice
    // (about 2^-24 * (|b| + 2^15 |a|) each); near planes move earlier and far
    // planes later by m = 2^-7 |a| + 2^-22 |b|, which covers that with room
    // to spare (2^-7 of a quantisation step), so culling stays as
    // conservative as the unfolded form.
    float ax = __fmul_rn(scx, r.inv.x), ay = __fmul_rn(scy, r.inv.y), az = __fmul_rn(scz, r.inv.z);
    const float bx0 = __fmaf_rn(n0.x, r.inv.x, -r.oinv.x);
    const float by0 = __fmaf_rn(n0.y, r.inv.y, -r.oinv.y);
    const float bz0 = __fmaf_rn(n0.z, r.inv.z, -r.oinv.z);
    const float mx = __fmaf_rn(fabsf(bx0), 0x1p-22f, __fmul_rn(fabsf(ax), 0x1p-7f));
    const float my = __fmaf_rn(fabsf(by0), 0x1p-22f, __fmul_rn(fabsf(ay), 0x1p-7f));
    const float mz = __fmaf_rn(fabsf(bz0), 0x1p-22f, __fmul_rn(fabsf(az), 0x1p-7f));
    const float fx0 = __fmaf_rn(-32768.0f, ax, bx0), fy0 = __fmaf_rn(-32768.0f, ay, by0);
    const float fz0 = __fmaf_rn(-32768.0f, az, bz0);
    const float bxn = __fsub_rn(fx0, mx), bxf = __fadd_rn(fx0, mx);
    const float byn = __fsub_rn(fy0, my), byf = __fadd_rn(fy0, my);
    const float bzn = __fsub_rn(fz0, mz), bzf = __fadd_rn(fz0, mz);
    // Near/far planes per axis chosen once per node by the ray octant
    // (d < 0: the hi plane is entered first).
    const bool sx = oct & 1u, sy = oct & 2u, sz = oct & 4u;
    uint32_t nx[2] = {sx ? __float_as_uint(n3.z) : __float_as_uint(n2.x), sx ? __float_as_uint(n3.w) : __float_as_uint(n2.y)};
    uint32_t fx[2] = {sx ? __float_as_uint(n2.x) : __float_as_uint(n3.z), sx ? __float_as_uint(n2.y) : __float_as_uint(n3.w)};
    uint32_t ny[2] = {sy ? __float_as_uint(n4.x) : __float_as_uint(n2.z), sy ? __float_as_uint(n4.y) : __float_as_uint(n2.w)};
    uint32_t fy[2] = {sy ? __float_as_uint(n2.z) : __float_as_uint(n4.x), sy ? __float_as_uint(n2.w) : __float_as_uint(n4.y)};
    uint32_t nz[2] = {sz ? __float_as_uint(n4.z) : __float_as_uint(n3.x), sz ? __float_as_uint(n4.w) : __float_as_uint(n3.y)};
    uint32_t fz[2] = {sz ? __float_as_uint(n3.x) : __float_as_uint(n4.z), sz ? __float_as_uint(n3.y) : __float_as_uint(n4.w)};
    // Meta bytes, four at a time: inner children (bits 4 and 3 set) get
    // their hit bit permuted by the octant; child_bits is the unary count.
    uint32_t bit_index[2], child_bits[2];
    const uint32_t oct4 = oct * 0x01010101u;
#pragma unroll
    for (int w = 0; w < 2; ++w) {
        uint32_t m4 = __float_as_uint(w ? n1.w : n1.z);
        uint32_t inner4 = (m4 & (m4 << 1)) & 0x10101010u;
        uint32_t perm = oct4 & ((inner4 >> 4) * 7u);
        bit_index[w] = (m4 ^ perm) & 0x1F1F1F1Fu;
        child_bits[w] = (m4 >> 5) & 0x07070707u;
    }
    // Box tests; a hit child contributes its unary count at its bit index
    // (empty slots have child_bits 0 and contribute nothing).  Building the
    // mask inside the unrolled loop, instead of looping over the hit bits
    // afterwards, removes a divergent loop of about 13 instructions per hit
    // child (8 % faster closest-hit traversal).
    uint32_t hitmask = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int w = c >> 2, b = c & 3;
        float tnx = __fmaf_rn(q2f(nx[w], b), ax, bxn), tfx = __fmaf_rn(q2f(fx[w], b), ax, bxf);
        float tny = __fmaf_rn(q2f(ny[w], b), ay, byn), tfy = __fmaf_rn(q2f(fy[w], b), ay, byf);
        float tnz = __fmaf_rn(q2f(nz[w], b), az, bzn), tfz = __fmaf_rn(q2f(fz[w], b), az, bzf);
        float tn = fmaxf(max3f(tnx, tny, tnz), r.tmin);
        float tf = fminf(min3f(tfx, tfy, tfz), tcur);
        const uint32_t contrib = __byte_perm(child_bits[w], 0u, 0x4440u | (uint32_t)b)
                                 << __byte_perm(bit_index[w], 0u, 0x4440u | (uint32_t)b);
        if (tn <= tf * kBoxSlack) hitmask |= contrib;
    }
    return hitmask;
}

// Persistent-warp traversal.  work[0] = next ray to hand out, work[1] =
// warps finished; the last warp to finish resets both, so the counters
// need no reset between launches that use them one after another.
template <bool CLOSEST, bool COUNT>
__global__ void __launch_bounds__(kBlock, 4) k_trace_bvh8(const float4* __restrict__ nodes,
                                                          const float4* __restrict__ tris,
                                                          const float4* __restrict__ rays, int4* __restrict__ results,
                                                          const uint32_t* __restrict__ ray_index, uint32_t n,
                                                          const uint32_t* __restrict__ n_dev,
                                                          uint32_t* __restrict__ work, uint32_t refill, uint32_t postpone) {
    const uint32_t count = load_count(n, n_dev);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint2 stack[kStack8];
    int sp = 0;
    uint32_t ri = kNoRay;
    // Lane state: idle (no ray), tracing, or done (result held in registers
    // until the next refill of the warp writes it, so the divergent write-out
    // runs once per refill instead of once per finished ray).
    enum : uint32_t { kIdle = 0, kTracing = 1, kDone = 2 };
    uint32_t state = kIdle;
    bool exhausted = false, found = false;
    RayT r;
    HitS h;
    uint2 ng = make_uint2(0u, 0u);  // node group: child base, hit bits 24..31 | imask 0..7
    uint32_t c_nodes = 0, c_tris = 0, c_rays = 0, c_iters = 0;
    for (;;) {
        // Refill non-tracing lanes with new rays (one atomic per warp).
        bool want = state != kTracing && !exhausted;
        uint32_t want_mask = __ballot_sync(0xffffffffu, want);
        uint32_t busy_mask = __ballot_sync(0xffffffffu, state == kTracing);
        if (want_mask != 0u && (__popc(want_mask) >= refill || busy_mask == 0u)) {
            if (state == kDone) {
                write_hit(results, ri, r, tris, h, found);
                state = kIdle;
            }
            uint32_t leader = __ffs(want_mask) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&work[0], __popc(want_mask));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (want) {
                uint32_t i = base + __popc(want_mask & lt_mask);
                if (i < count) {
                    uint32_t idx = ray_index ? ray_index[i] : i;
                    float4 r0 = rays[2 * idx + 0];
                    float4 r1 = rays[2 * idx + 1];
                    if (!(r1.w >= r0.w)) {  // empty interval: miss, lane stays idle
                        write_miss(results, idx);
                    } else {
                        ri = idx;
                        state = kTracing;
                        r = setup_ray(r0, r1);
                        h = HitS{r1.w, 0xFFFFFFFFu, 0u};
                        found = false;
                        sp = 0;
                        ng = make_uint2(0u, 0x80000000u);  // root as the only child of a virtual group
                    }
                } else {
                    exhausted = true;
                }
            }
        }
        const uint32_t busy = __ballot_sync(0xffffffffu, state == kTracing);
        if (__ballot_sync(0xffffffffu, state != kIdle || !exhausted) == 0u) break;
        if (COUNT && lane == 0) ++c_iters;
        if (state != kTracing) continue;

        // The current group is either a node group (hit bits 24..31) or a
        // triangle group popped from the stack (bits 0..23, base in x).
        uint32_t tri_base = 0, tg = 0;
        if (ng.y > 0x00FFFFFFu) {
            // One node: pick the nearest child of the current group.
            uint32_t bit = 31u - __clz(ng.y);
            ng.y &= ~(1u << bit);
            uint32_t slot = (bit - 24u) ^ r.oct;
            uint32_t node = ng.x + __popc(ng.y & ((1u << slot) - 1u) & 0xFFu);
            if (ng.y > 0x00FFFFFFu) {
                if (sp < kStack8) {
                    stack[sp++] = ng;
                } else {
                    raise_status(kErrBounds);
                }
            }
            uint32_t child_base, imask;
            if (COUNT) ++c_nodes;
            uint32_t hitmask = intersect_node8(nodes + 5 * (size_t)node, r, h.t, child_base, tri_base, imask);
            ng = make_uint2(child_base, (hitmask & 0xFF000000u) | imask);
            tg = hitmask & 0x00FFFFFFu;
        } else {
            tri_base = ng.x;
            tg = ng.y;
            ng = make_uint2(0u, 0u);
        }
        // Postpone a node's triangles while few lanes of the warp have any
        // and more nodes remain: they wait on the stack as a triangle group.
        if (postpone != 0u) {
            uint32_t with_tris = __ballot_sync(busy, tg != 0u);
            if (tg != 0u && ng.y > 0x00FFFFFFu && (uint32_t)__popc(with_tris) < postpone && sp < kStack8) {
                stack[sp++] = make_uint2(tri_base, tg);
                tg = 0;
            }
        }
        bool finished = false;
        while (tg != 0u) {
            uint32_t tb = __ffs(tg) - 1u;
            tg &= tg - 1u;
            if (COUNT) ++c_tris;
            if (intersect_tri(r, tris, tri_base + tb, h)) {
                found = true;
                if (!CLOSEST) {
                    finished = true;
                    break;
                }
            }
        }
        if (!finished && ng.y <= 0x00FFFFFFu) {
            if (sp == 0) {
                finished = true;
            } else {
                ng = stack[--sp];
            }
        }
        if (finished) {
            state = kDone;
            if (COUNT) ++c_rays;
        }
    }
    if (COUNT) add_counts(c_nodes, c_tris, c_rays, c_iters);
    // Last warp out resets the work counters for the next launch.
    if (lane == 0) {
        uint32_t warps = gridDim.x * (blockDim.x / 32);
        __threadfence();
        if (atomicAdd(&work[1], 1u) == warps - 1u) {
            work[0] = 0u;
            work[1] = 0u;
            __threadfence();
        }
    }
}

// ------------------------------------ BVH8 with warp-cooperative triangles
// Ray fields the triangle test reads, kept in shared memory so that any
// lane of the warp can test a triangle against any other lane's ray.
struct alignas(16) RayS {
    float ox, oy, oz, tmin;
    float sx, sy, sz;
    uint32_t k;  // kx | ky << 2 | kz << 4
};

__device__ __forceinline__ RayS ray_shared(const RayT& r) {
    RayS s;
    s.ox = r.o.x;
    s.oy = r.o.y;
    s.oz = r.o.z;
    s.tmin = r.tmin;
    s.sx = r.sx;
    s.sy = r.sy;
    s.sz = r.sz;
    s.k = (uint32_t)r.kx | ((uint32_t)r.ky << 2) | ((uint32_t)r.kz << 4);
    return s;
}

__device__ __forceinline__ Uvw tri_uvw(const RayS& s, const float4& a4, const float4& b4, const float4& c4) {
    return tri_uvw(mk(s.ox, s.oy, s.oz), (int)(s.k & 3u), (int)((s.k >> 2) & 3u), (int)(s.k >> 4), s.sx, s.sy, s.sz,
                   a4, b4, c4);
}

// The closest-hit order as one 64-bit key: distance bits mapped to an
// order-preserving unsigned (-0 folded onto +0, so equal distances compare
// equal), then the global triangle index.  atomicMin over these keys picks
// the hit of the sequential rule (smaller t, then smaller index) in any
// order of arrival.
__device__ __forceinline__ unsigned long long hit_key(float t, uint32_t key) {
    uint32_t b = __float_as_uint(__fadd_rn(t, 0.0f));
    b ^= (uint32_t)((int32_t)b >> 31) | 0x80000000u;
    return ((unsigned long long)b << 32) | key;
}

__device__ __forceinline__ float hit_key_t(unsigned long long k) {
    uint32_t b = (uint32_t)(k >> 32);
    b = (b & 0x80000000u) ? (b ^ 0x80000000u) : ~b;
    return __uint_as_float(b);
}

constexpr uint32_t kRecBits = 27;  // task word: lane << 27 | triangle record
constexpr int kRing = 1024;        // per-warp ring of pending triangle tests (power of two)

// Same traversal as k_trace_bvh8, except that triangle tests are shared by
// the warp: each node step appends its lanes' (lane, triangle) pairs to a
// ring in shared memory, and the warp tests the ring 32 pairs at a time,
// each result folded into the owner's best hit key with a shared atomicMin;
// the test whose key is the owner's best after its round stores the hit's
// primitive, geometry, barycentrics and t beside it, so a finished lane
// writes its RayResult from shared memory (no reload of the winning
// triangle at write-out: 2 % faster any hit).  Tests are batched across node steps: the ring is tested once `batch` or
// more pairs are pending (in whole passes of 32 when 32 or more are), and
// entirely once the lanes waiting on their own tests plus the idle lanes
// would fill a refill, or no lane has nodes left.  A loop iteration takes up
// to `steps` node steps per lane, stopping at the first node that hands the
// lane triangles, so the per-iteration work (refill check, votes, scan,
// test decision) is shared by several node steps.  A lane's ray finishes
// only when its traversal is exhausted (any hit: when it has a hit) and all
// of its own tests have run, so a ring entry never outlives its ray.  The
// deferred tests leave tcur larger for a few node steps (culling stays
// conservative: tcur only shrinks), which costs about 1 % more node steps
// and saves most of the partly empty test passes (batch 1: test every
// step).  A lane appends at most one node's 24 triangles per iteration, so
// at most 31 + 32 * 24 pairs are pending after an append.
template <bool CLOSEST, bool COUNT>
__global__ void __launch_bounds__(kBlock, 4) k_trace_bvh8_coop(
    const float4* __restrict__ nodes, const float4* __restrict__ tris, const float4* __restrict__ rays,
    int4* __restrict__ results, const uint32_t* __restrict__ ray_index, uint32_t n,
    const uint32_t* __restrict__ n_dev, uint32_t* __restrict__ work,
    uint32_t refill, uint32_t batch, uint32_t steps) {
    __shared__ RayS s_ray[kBlock];
    __shared__ unsigned long long s_best[kBlock];
    __shared__ uint4 s_hit[kBlock];  // winning hit: primId, geomId, packed barycentrics, t
    __shared__ uint32_t s_task[kBlock / 32][kRing];
    const uint32_t count = load_count(n, n_dev);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t wbase = threadIdx.x & ~31u;
    uint32_t* const task = s_task[threadIdx.x >> 5];
    uint2 stack[kStack8];
    int sp = 0;
    uint32_t ri = kNoRay;
    enum : uint32_t { kIdle = 0, kTracing = 1, kDone = 2 };
    uint32_t state = kIdle;
    bool exhausted = false;
    RayT r;
    float tcur = 0.0f;
    uint2 ng = make_uint2(0u, 0u);
    // Ring counters (absolute, wrapped by the ring mask; equal in all
    // lanes): pairs [tested, appended) are pending.  my_end: one past this
    // lane's last appended pair.
    uint32_t tested = 0, appended = 0, my_end = 0;
    uint32_t c_nodes = 0, c_tris = 0, c_rays = 0, c_iters = 0;
    for (;;) {
        bool want = state != kTracing && !exhausted;
        uint32_t want_mask = __ballot_sync(0xffffffffu, want);
        uint32_t busy_mask = __ballot_sync(0xffffffffu, state == kTracing);
        if (want_mask != 0u && (__popc(want_mask) >= refill || busy_mask == 0u)) {
            if (state == kDone) {
                const unsigned long long best = s_best[threadIdx.x];
                if ((uint32_t)best == 0xFFFFFFFFu) {
                    write_miss(results, ri);
                } else {
                    const uint4 hh = s_hit[threadIdx.x];
                    results[ri] = make_int4((int)hh.x, (int)hh.y, (int)hh.w, (int)hh.z);
                }
                state = kIdle;
            }
            uint32_t leader = __ffs(want_mask) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&work[0], __popc(want_mask));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (want) {
                uint32_t i = base + __popc(want_mask & lt_mask);
                if (i < count) {
                    uint32_t idx = ray_index ? ray_index[i] : i;
                    float4 r0 = rays[2 * idx + 0];
                    float4 r1 = rays[2 * idx + 1];
                    if (!(r1.w >= r0.w)) {  // empty interval: miss, lane stays idle
                        write_miss(results, idx);
                    } else {
                        ri = idx;
                        state = kTracing;
                        r = setup_ray(r0, r1);
                        s_ray[threadIdx.x] = ray_shared(r);
                        s_best[threadIdx.x] = hit_key(r1.w, 0xFFFFFFFFu);
                        tcur = r1.w;
                        sp = 0;
                        ng = make_uint2(0u, 0x80000000u);
                    }
                } else {
                    exhausted = true;
                }
            }
            want_mask = 0u;  // refilled (or out of rays)
        }
        if (__ballot_sync(0xffffffffu, state != kIdle || !exhausted) == 0u) break;
        if (COUNT && lane == 0) ++c_iters;

        // Up to `steps` node steps; a lane stops stepping at the first node
        // that hands it triangles (at most one group of 24 per iteration).
        uint32_t tri_base = 0, tg = 0;
        for (uint32_t st = 0; st < steps; ++st) {
            const bool go = state == kTracing && ng.y > 0x00FFFFFFu && tg == 0u;
            if (st != 0u && !__any_sync(0xffffffffu, go)) break;
            if (go) {
                uint32_t bit = 31u - __clz(ng.y);
                ng.y &= ~(1u << bit);
                uint32_t slot = (bit - 24u) ^ r.oct;
                uint32_t node = ng.x + __popc(ng.y & ((1u << slot) - 1u) & 0xFFu);
                if (ng.y > 0x00FFFFFFu) {
                    if (sp < kStack8) {
                        stack[sp++] = ng;
                    } else {
                        raise_status(kErrBounds);
                    }
                }
                uint32_t child_base, imask;
                if (COUNT) ++c_nodes;
                uint32_t hitmask = intersect_node8(nodes + 5 * (size_t)node, r, tcur, child_base, tri_base, imask);
                ng = make_uint2(child_base, (hitmask & 0xFF000000u) | imask);
                tg = hitmask & 0x00FFFFFFu;
            }
            if (state == kTracing && ng.y <= 0x00FFFFFFu && sp > 0) ng = stack[--sp];
        }

        // Append this step's pairs: exclusive scan of the per-lane counts.
        const uint32_t cnt = __popc(tg);
        uint32_t incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += v;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        if (cnt != 0u) {
            uint32_t pos = appended + incl - cnt;
            const uint32_t owner = lane << kRecBits;
            while (tg != 0u) {
                uint32_t tb = __ffs(tg) - 1u;
                tg &= tg - 1u;
                task[pos++ & (kRing - 1)] = owner | (tri_base + tb);
            }
            my_end = pos;
            if (COUNT) c_tris += cnt;
        }
        appended += total;

        // A tracing lane without nodes left waits for its own tests.
        const bool waiting = state == kTracing && ng.y <= 0x00FFFFFFu;
        const uint32_t walk_mask = __ballot_sync(0xffffffffu, state == kTracing && !waiting);
        const uint32_t wait_mask = __ballot_sync(0xffffffffu, waiting && (int32_t)(my_end - tested) > 0);
        const uint32_t pend = appended - tested;
        uint32_t nflush = 0;
        if (pend != 0u) {
            if (walk_mask == 0u || batch <= 1u || (uint32_t)__popc(wait_mask | want_mask) >= refill)
                nflush = pend;
            else if (pend >= batch)
                nflush = pend >= 32u ? (pend & ~31u) : pend;
        }
        if (nflush != 0u) {
            __syncwarp();
            for (uint32_t j0 = 0; j0 < nflush; j0 += 32u) {
                const uint32_t j = j0 + lane;
                bool cand = false;
                unsigned long long hk = 0;
                uint32_t o = 0;
                uint4 hh = make_uint4(0u, 0u, 0u, 0u);
                if (j < nflush) {
                    const uint32_t w = task[(tested + j) & (kRing - 1)];
                    o = wbase + (w >> kRecBits);
                    const uint32_t rec = w & ((1u << kRecBits) - 1u);
                    const RayS rs = s_ray[o];
                    float4 a4 = __ldg(&tris[3 * rec + 0]);
                    float4 b4 = __ldg(&tris[3 * rec + 1]);
                    float4 c4 = __ldg(&tris[3 * rec + 2]);
                    Uvw q = tri_uvw(rs, a4, b4, c4);
                    if (q.edge_ok && q.det != 0.0f) {
                        float t = __fdiv_rn(q.T, q.det);
                        if (t >= rs.tmin) {
                            // A stale read can only be larger than the current
                            // best, so skipping on it is safe.
                            hk = hit_key(t, __float_as_uint(c4.w));
                            if (hk < s_best[o]) {
                                atomicMin(&s_best[o], hk);
                                cand = true;
                                const float u = __fdiv_rn(q.V, q.det), v = __fdiv_rn(q.W, q.det);
                                hh = make_uint4(__float_as_uint(a4.w), __float_as_uint(b4.w), pack_unorm2x16(u, v),
                                                __float_as_uint(t));
                            }
                        }
                    }
                }
                // The candidate whose key is the owner's best after this
                // round records the hit's fields (keys are unique).
                __syncwarp();
                if (cand && s_best[o] == hk) s_hit[o] = hh;
            }
            __syncwarp();
            tested += nflush;
        }

        if (state == kTracing) {
            const unsigned long long best = s_best[threadIdx.x];
            tcur = hit_key_t(best);
            bool stop = waiting;
            if (!CLOSEST && (uint32_t)best != 0xFFFFFFFFu) {
                stop = true;  // any hit: no more node steps
                ng.y = 0u;
                sp = 0;
            }
            if (stop && (int32_t)(my_end - tested) <= 0) {
                state = kDone;
                if (COUNT) ++c_rays;
            }
        }
    }
    if (COUNT) add_counts(c_nodes, c_tris, c_rays, c_iters);
    if (lane == 0) {
        uint32_t warps = gridDim.x * (blockDim.x / 32);
        __threadfence();
        if (atomicAdd(&work[1], 1u) == warps - 1u) {
            work[0] = 0u;
            work[1] = 0u;
            __threadfence();
        }
    }
}

// Work-counter slots (16 u32 apart) handed out round robin, so concurrent
// traces on different streams do not share a counter.
static std::atomic<uint32_t> g_slot{0};
// Resident blocks per SM: [closest] for the per-lane kernel, [2 + closest]
// for the cooperative one.
static int g_blocks_per_sm[4] = {0, 0, 0, 0};
static int g_num_sms = 0;
static uint32_t g_refill = 8;

void set_trace_refill(uint32_t refill) { g_refill = refill < 1 ? 1 : (refill > 32 ? 32 : refill); }
static uint32_t g_postpone = 0;
void set_trace_postpone(uint32_t lanes) { g_postpone = lanes > 32 ? 32 : lanes; }
// Cooperative-test batch and node steps per loop iteration, [0] for any-hit
// rays, [1] for closest-hit rays.  Any-hit rays test their triangles after
// every iteration of three node steps (a ray stops at its first hit, so
// deferring tests only adds node steps), closest-hit rays batch 24 pairs
// over iterations of two steps: measured on the courtyard's bounce-1 rays
// (1.4 % / 0.6 % faster than the shared batch 16, steps 2) and its frames
// (25.28 against 25.38 ms).
static uint32_t g_batch[2] = {1, 24};
static uint32_t g_steps[2] = {3, 2};
void set_trace_steps(uint32_t steps, bool closest) {
    g_steps[closest ? 1 : 0] = steps < 1 ? 1 : (steps > 8 ? 8 : steps);
}
uint32_t get_trace_steps(bool closest) { return g_steps[closest ? 1 : 0]; }
void set_trace_batch(uint32_t pairs, bool closest) {
    g_batch[closest ? 1 : 0] = pairs < 1 ? 1 : (pairs > 32 ? 32 : pairs);
}
uint32_t get_trace_batch(bool closest) { return g_batch[closest ? 1 : 0]; }
static bool g_coop = true;
void set_trace_coop(bool on) { g_coop = on; }
bool get_trace_coop() { return g_coop; }
uint32_t get_trace_refill() { return g_refill; }
static bool g_count = false;
void set_trace_count(bool on) { g_count = on; }
bool get_trace_count() { return g_count; }

// SM count and resident blocks of the persistent kernel (host queries that
// must not run inside a stream capture; the renderer calls this first).
cudaError_t trace_prepare() {
    if (g_num_sms != 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks_per_sm[0], k_trace_bvh8<false, false>, kBlock, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks_per_sm[1], k_trace_bvh8<true, false>, kBlock, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks_per_sm[2], k_trace_bvh8_coop<false, false>, kBlock,
                                                          0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks_per_sm[3], k_trace_bvh8_coop<true, false>, kBlock,
                                                          0);
    if (e == cudaSuccess) g_num_sms = sms;
    return e;
}

cudaError_t trace_counters(uint64_t out[4], bool reset) {
    unsigned long long v[4];
    cudaError_t e = cudaMemcpyFromSymbol(v, g_counts, sizeof(v));
    if (e != cudaSuccess) return e;
    for (int i = 0; i < 4; ++i) out[i] = v[i];
    if (reset) {
        unsigned long long z[4] = {0, 0, 0, 0};
        e = cudaMemcpyToSymbol(g_counts, z, sizeof(z));
    }
    return e;
}
uint32_t get_trace_postpone() { return g_postpone; }

cudaError_t launch_trace(const SceneDevice& sc, int kind, const wfpt_ray* rays, wfpt_hit* results,
                         const uint32_t* ray_index, uint32_t n, const uint32_t* n_dev, int closest,
                         cudaStream_t s, uint32_t* own_work) {
    if (n == 0) return cudaSuccess;
    // A scene built without this BVH kind has no buffers for it.
    if (kind == WFPT_BVH8_Q8 ? (!sc.bvh8_nodes || !sc.bvh8_tris) : (!sc.bvh2_nodes || !sc.bvh2_tris))
        return cudaErrorInvalidValue;
    unsigned grid = (n + kBlock - 1) / kBlock;
    const float4* rr = reinterpret_cast<const float4*>(rays);
    int4* out = reinterpret_cast<int4*>(results);
    if (kind == WFPT_BVH8_Q8) {
        if (g_num_sms == 0) {
            cudaError_t e = trace_prepare();
            if (e != cudaSuccess) return e;
        }
        // The cooperative kernel packs a triangle record into 27 bits.
        const bool coop = g_coop && sc.bvh8_num_tris < (1u << kRecBits);
        unsigned pgrid = (unsigned)(g_num_sms * g_blocks_per_sm[(coop ? 2 : 0) + (closest ? 1 : 0)]);
        if (pgrid == 0) pgrid = 1;
        if (grid < pgrid) pgrid = grid;
        uint32_t* work = own_work ? own_work : sc.work + 16 * (g_slot.fetch_add(1) % kWorkSlots);
        if (coop) {
            auto k8 = closest ? (g_count ? k_trace_bvh8_coop<true, true> : k_trace_bvh8_coop<true, false>)
                              : (g_count ? k_trace_bvh8_coop<false, true> : k_trace_bvh8_coop<false, false>);
            k8<<<pgrid, kBlock, 0, s>>>(sc.bvh8_nodes, sc.bvh8_tris, rr, out, ray_index, n, n_dev, work, g_refill,
                                        g_batch[closest ? 1 : 0], g_steps[closest ? 1 : 0]);
        } else {
            auto k8 = closest ? (g_count ? k_trace_bvh8<true, true> : k_trace_bvh8<true, false>)
                              : (g_count ? k_trace_bvh8<false, true> : k_trace_bvh8<false, false>);
            k8<<<pgrid, kBlock, 0, s>>>(sc.bvh8_nodes, sc.bvh8_tris, rr, out, ray_index, n, n_dev, work, g_refill,
                                        g_postpone);
        }
    } else {
        auto k2 = closest ? (g_count ? k_trace_bvh2<true, true> : k_trace_bvh2<true, false>)
                          : (g_count ? k_trace_bvh2<false, true> : k_trace_bvh2<false, false>);
        k2<<<grid, kBlock, 0, s>>>(sc.bvh2_nodes, sc.bvh2_tris, rr, out, ray_index, n, n_dev);
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace wfpt
