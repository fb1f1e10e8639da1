// Software BVH traversal: replaces trace.comp's rayQuery (trace.comp:50-84)
// on a GPU without RT cores.
//
// Plain form  (WFPT_BVH2_FP32): binary BVH, each 64-byte node holds both
//   children's FP32 boxes; while-while traversal with a per-thread stack.
// Chosen form (WFPT_BVH8_Q8):   8-wide BVH, 80-byte nodes with an FP32
//   origin, per-axis power-of-two scales and 8-bit child boxes rounded
//   outward; children visited in ray-octant order, node groups on the stack
//   (Ylitie, Karras, Laine: "Efficient Incoherent Ray Traversal on GPUs
//   Through Compressed Wide BVHs", HPG 2017).
// Both use the watertight ray/triangle test of Woop, Benthin and Wald
// (JCGT 2013), evaluated without FMA contraction, and the same closest-hit
// rule (smallest t, ties to the smaller global triangle index), so both
// forms return identical hits.
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

struct RayT {
    f3 o;
    f3 d;
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
    r.d = mk(r1.x, r1.y, r1.z);
    r.tmin = r0.w;
    r.inv = mk(safe_inv(r.d.x), safe_inv(r.d.y), safe_inv(r.d.z));
    r.oinv = mul(r.o, r.inv);
    float ax = fabsf(r.d.x), ay = fabsf(r.d.y), az = fabsf(r.d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (comp(r.d, kz) < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    float dz = comp(r.d, kz);
    r.sx = __fdiv_rn(comp(r.d, kx), dz);
    r.sy = __fdiv_rn(comp(r.d, ky), dz);
    r.sz = __fdiv_rn(1.0f, dz);
    // Sign bits (not d < 0): -0.0 has a negative reciprocal in safe_inv, and
    // the BVH8 near/far plane choice must agree with the sign of inv.
    r.oct = (__float_as_uint(r.d.x) >> 31) | ((__float_as_uint(r.d.y) >> 31) << 1) |
            ((__float_as_uint(r.d.z) >> 31) << 2);
    return r;
}

struct Hit {
    float t;
    uint32_t key;  // global triangle index of the current best hit
    int prim, geom;
    float u, v;
};

// Watertight test; on acceptance updates `h` and returns true.
__device__ __forceinline__ bool intersect_tri(const RayT& r, const float4* __restrict__ tris, uint32_t ti,
                                              Hit& h) {
    float4 a4 = __ldg(&tris[3 * ti + 0]);
    float4 b4 = __ldg(&tris[3 * ti + 1]);
    float4 c4 = __ldg(&tris[3 * ti + 2]);
    f3 A = sub(mk(a4.x, a4.y, a4.z), r.o);
    f3 B = sub(mk(b4.x, b4.y, b4.z), r.o);
    f3 C = sub(mk(c4.x, c4.y, c4.z), r.o);
    float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    float Ax = __fsub_rn(comp(A, r.kx), __fmul_rn(r.sx, Akz));
    float Ay = __fsub_rn(comp(A, r.ky), __fmul_rn(r.sy, Akz));
    float Bx = __fsub_rn(comp(B, r.kx), __fmul_rn(r.sx, Bkz));
    float By = __fsub_rn(comp(B, r.ky), __fmul_rn(r.sy, Bkz));
    float Cx = __fsub_rn(comp(C, r.kx), __fmul_rn(r.sx, Ckz));
    float Cy = __fsub_rn(comp(C, r.ky), __fmul_rn(r.sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double cxby = (double)Cx * (double)By, cybx = (double)Cy * (double)Bx;
        U = (float)(cxby - cybx);
        double axcy = (double)Ax * (double)Cy, aycx = (double)Ay * (double)Cx;
        V = (float)(axcy - aycx);
        double bxay = (double)Bx * (double)Ay, byax = (double)By * (double)Ax;
        W = (float)(bxay - byax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    float Az = __fmul_rn(r.sz, Akz), Bz = __fmul_rn(r.sz, Bkz), Cz = __fmul_rn(r.sz, Ckz);
    float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    float t = __fdiv_rn(T, det);
    if (!(t >= r.tmin)) return false;
    uint32_t key = __float_as_uint(c4.w);
    if (!(t < h.t || (t == h.t && key < h.key))) return false;
    h.t = t;
    h.key = key;
    h.prim = __float_as_int(a4.w);
    h.geom = __float_as_int(b4.w);
    h.u = __fdiv_rn(V, det);
    h.v = __fdiv_rn(W, det);
    return true;
}

__device__ __forceinline__ void write_hit(int4* __restrict__ results, uint32_t ri, const Hit& h, bool found) {
    int4 out;
    if (found) {
        out = make_int4(h.prim, h.geom, __float_as_int(h.t), (int)pack_unorm2x16(h.u, h.v));
    } else {
        out = make_int4(-1, -1, __float_as_int(-1.0f), 0);
    }
    results[ri] = out;
}

// ------------------------------------------------------------ BVH2 (plain)
__device__ __forceinline__ void box2(const RayT& r, float lox, float hix, float loy, float hiy, float loz,
                                     float hiz, float tcur, float& tnear, bool& hit) {
    float x0 = __fmaf_rn(lox, r.inv.x, -r.oinv.x), x1 = __fmaf_rn(hix, r.inv.x, -r.oinv.x);
    float y0 = __fmaf_rn(loy, r.inv.y, -r.oinv.y), y1 = __fmaf_rn(hiy, r.inv.y, -r.oinv.y);
    float z0 = __fmaf_rn(loz, r.inv.z, -r.oinv.z), z1 = __fmaf_rn(hiz, r.inv.z, -r.oinv.z);
    float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), r.tmin));
    float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tcur));
    tnear = tn;
    hit = tn <= tf * kBoxSlack;
}

template <bool CLOSEST>
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
    Hit h;
    h.t = r1.w;
    h.key = 0xFFFFFFFFu;
    bool found = false;
    if (!(r1.w >= r0.w)) {  // tmax < tmin (or NaN): empty interval
        write_hit(results, ri, h, false);
        return;
    }
    RayT r = setup_ray(r0, r1);
    int stack[kStack2];
    int sp = 0;
    int node = 0;
    bool done = false;
    while (!done) {
        // Inner nodes.
        while (node >= 0) {
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
    write_hit(results, ri, h, found);
}

// --------------------------------------------------------- BVH8 (chosen)
__device__ __forceinline__ uint32_t byte_of(uint32_t w, int b) { return (w >> (8 * b)) & 0xFFu; }

// Byte b of w as an exact float: the byte is permuted into the mantissa of
// 2^23 (bits 0x4B000000), then 2^23 is subtracted -- one PRMT and one FADD
// instead of an integer-to-float conversion.
__device__ __forceinline__ float q2f(uint32_t w, int b) {
    return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7650u | (uint32_t)b)), 8388608.0f);
}

template <bool CLOSEST>
__global__ void __launch_bounds__(kBlock) k_trace_bvh8(const float4* __restrict__ nodes,
                                                       const float4* __restrict__ tris,
                                                       const float4* __restrict__ rays, int4* __restrict__ results,
                                                       const uint32_t* __restrict__ ray_index, uint32_t n,
                                                       const uint32_t* __restrict__ n_dev) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= load_count(n, n_dev)) return;
    uint32_t ri = ray_index ? ray_index[i] : i;
    float4 r0 = rays[2 * ri + 0];
    float4 r1 = rays[2 * ri + 1];
    Hit h;
    h.t = r1.w;
    h.key = 0xFFFFFFFFu;
    bool found = false;
    if (!(r1.w >= r0.w)) {
        write_hit(results, ri, h, false);
        return;
    }
    RayT r = setup_ray(r0, r1);
    const uint32_t oct = r.oct;
    uint2 stack[kStack8];
    int sp = 0;
    // Node group: x = child base index, y = node hit bits (24..31) | imask (0..7).
    uint2 ng = make_uint2(0u, 0x80000000u);
    for (;;) {
        uint32_t bit = 31u - __clz(ng.y);
        ng.y &= ~(1u << bit);
        uint32_t slot = (bit - 24u) ^ oct;
        uint32_t node = ng.x + __popc(ng.y & ((1u << slot) - 1u) & 0xFFu);
        if (ng.y > 0x00FFFFFFu) {
            if (sp < kStack8) {
                stack[sp++] = ng;
            } else {
                raise_status(kErrBounds);
            }
        }
        const float4* nd = nodes + 5 * (size_t)node;
        float4 n0 = __ldg(nd + 0);
        float4 n1 = __ldg(nd + 1);
        float4 n2 = __ldg(nd + 2);
        float4 n3 = __ldg(nd + 3);
        float4 n4 = __ldg(nd + 4);
        uint32_t ew = __float_as_uint(n0.w);
        float scx = __uint_as_float((ew & 0xFFu) << 23);
        float scy = __uint_as_float(((ew >> 8) & 0xFFu) << 23);
        float scz = __uint_as_float(((ew >> 16) & 0xFFu) << 23);
        uint32_t imask = ew >> 24;
        // Slab distance = q * (scale*inv) + (p - o) * inv.
        float ax = __fmul_rn(scx, r.inv.x), ay = __fmul_rn(scy, r.inv.y), az = __fmul_rn(scz, r.inv.z);
        float bx = __fmaf_rn(n0.x, r.inv.x, -r.oinv.x);
        float by = __fmaf_rn(n0.y, r.inv.y, -r.oinv.y);
        float bz = __fmaf_rn(n0.z, r.inv.z, -r.oinv.z);
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
        uint32_t hitmask = 0;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int w = c >> 2, b = c & 3;
            float tnx = __fmaf_rn(q2f(nx[w], b), ax, bx), tfx = __fmaf_rn(q2f(fx[w], b), ax, bx);
            float tny = __fmaf_rn(q2f(ny[w], b), ay, by), tfy = __fmaf_rn(q2f(fy[w], b), ay, by);
            float tnz = __fmaf_rn(q2f(nz[w], b), az, bz), tfz = __fmaf_rn(q2f(fz[w], b), az, bz);
            float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, r.tmin));
            float tf = fminf(fminf(tfx, tfy), fminf(tfz, h.t));
            if (tn <= tf * kBoxSlack) hitmask |= byte_of(child_bits[w], b) << byte_of(bit_index[w], b);
        }
        uint32_t tri_base = __float_as_uint(n1.y);
        ng = make_uint2(__float_as_uint(n1.x), (hitmask & 0xFF000000u) | imask);
        uint32_t tg = hitmask & 0x00FFFFFFu;
        bool stop = false;
        while (tg != 0u) {
            uint32_t tb = __ffs(tg) - 1u;
            tg &= tg - 1u;
            if (intersect_tri(r, tris, tri_base + tb, h)) {
                found = true;
                if (!CLOSEST) {
                    stop = true;
                    break;
                }
            }
        }
        if (stop) break;
        if (ng.y <= 0x00FFFFFFu) {
            if (sp == 0) break;
            ng = stack[--sp];
        }
    }
    write_hit(results, ri, h, found);
}

cudaError_t launch_trace(const SceneDevice& sc, int kind, const wfpt_ray* rays, wfpt_hit* results,
                         const uint32_t* ray_index, uint32_t n, const uint32_t* n_dev, int closest,
                         cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    unsigned grid = (n + kBlock - 1) / kBlock;
    const float4* rr = reinterpret_cast<const float4*>(rays);
    int4* out = reinterpret_cast<int4*>(results);
    if (kind == WFPT_BVH8_Q8) {
        if (closest)
            k_trace_bvh8<true><<<grid, kBlock, 0, s>>>(sc.bvh8_nodes, sc.bvh8_tris, rr, out, ray_index, n, n_dev);
        else
            k_trace_bvh8<false><<<grid, kBlock, 0, s>>>(sc.bvh8_nodes, sc.bvh8_tris, rr, out, ray_index, n, n_dev);
    } else {
        if (closest)
            k_trace_bvh2<true><<<grid, kBlock, 0, s>>>(sc.bvh2_nodes, sc.bvh2_tris, rr, out, ray_index, n, n_dev);
        else
            k_trace_bvh2<false><<<grid, kBlock, 0, s>>>(sc.bvh2_nodes, sc.bvh2_tris, rr, out, ray_index, n, n_dev);
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace wfpt
