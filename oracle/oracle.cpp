// Test infrastructure: CPU oracle for the wavefront stage chain.
//
// A scalar restatement of the reference compute shaders
// (shaders/glsl/WaveFrontPathTracer/*.comp) and of the host orchestration
// (projects/WaveFrontPathTracer/Renderer/Renderer.cpp), used only by the
// tests, by smoke checks and as the timed CPU baseline.  It is never part of
// the product path.  Built with -ffp-contract=off so that every float
// expression rounds exactly as written (GLSL shaders are written the same
// way, one rounding per operation).
//
// Parity status: pinned to the reference's own sources.  The shaders of
// every stage except the rayQuery traversal, the pixel-table loops and the
// camera header compile for the CPU (oracle/ref_build.py -> oracle/_ref);
// tests/test_oracle_ref_cpu.py and tests/golden/ref_vectors.npz hold this
// restatement to their outputs.  The traversal is checked by the FP64
// oracle below; the sort's definition is the stable order by key.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

struct ORay {
    float ox, oy, oz, tmin, dx, dy, dz, tmax;
};
struct OHit {
    int32_t prim, geom;
    float t;
    uint32_t bary;
};
struct OGeom {
    uint64_t vertex_addr, index_addr;  // host pointers here
};

extern "C" int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// ------------------------------------------------------------ vec3 shim
struct V3 {
    float x, y, z;
};
static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float len3(V3 a) { return std::sqrt(dot3(a, a)); }
static inline V3 normalize3(V3 a) { return a / len3(a); }
static inline V3 faceforward3(V3 n, V3 i, V3 nref) { return dot3(nref, i) < 0.0f ? n : v3(-n.x, -n.y, -n.z); }
static inline float clamp01(float x) { return std::fmin(std::fmax(x, 0.0f), 1.0f); }

// ------------------------------------------------------------- initSeeds
// initSeeds.comp:7-19, :36-40.
static uint32_t tea(uint32_t val0, uint32_t val1, uint32_t rounds) {
    uint32_t v0 = val0, v1 = val1, s0 = 0u;
    for (uint32_t n = 0; n < rounds; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

extern "C" void orc_init_seeds(uint32_t* seeds, uint32_t n, int frame_index) {
    for (uint32_t i = 0; i < n; ++i) seeds[i] = tea(i, (uint32_t)frame_index, 16);
}

// ------------------------------------------------------------ PixelTable
// Ray/PixelTable.cpp:33-93.
extern "C" void orc_pixel_table(int w, int h, int32_t* idxtopos, int32_t* postoidx) {
    int idx = 0;
    int bheight = h & ~7, bwidth = w & ~7;
    int maxdim = (bwidth > bheight) ? bwidth : bheight;
    maxdim |= maxdim >> 1;
    maxdim |= maxdim >> 2;
    maxdim |= maxdim >> 4;
    maxdim |= maxdim >> 8;
    maxdim |= maxdim >> 16;
    maxdim = (maxdim + 1) >> 1;
    int width8 = bwidth >> 3, height8 = bheight >> 3;
    for (long long i = 0; i < (long long)maxdim * maxdim; i++) {
        int tx = 0, ty = 0, bit = 1;
        long long val = i;
        while (val) {
            if (val & 1) tx |= bit;
            if (val & 2) ty |= bit;
            bit += bit;
            val >>= 2;
        }
        if (tx < width8 && ty < height8) {
            for (int inner = 0; inner < 64; inner++) {
                int ix = ((inner & 1) >> 0) | ((inner & 4) >> 1) | ((inner & 16) >> 2);
                int iy = ((inner & 2) >> 1) | ((inner & 8) >> 2) | ((inner & 32) >> 3);
                int pos = (ty * 8 + iy) * w + (tx * 8 + ix);
                postoidx[pos] = idx;
                idxtopos[idx++] = pos;
            }
        }
    }
    for (int px = 0; px < bwidth; px++)
        for (int py = bheight; py < h; py++) {
            int pos = px + py * w;
            postoidx[pos] = idx;
            idxtopos[idx++] = pos;
        }
    for (int py = 0; py < h; py++)
        for (int px = bwidth; px < w; px++) {
            int pos = px + py * w;
            postoidx[pos] = idx;
            idxtopos[idx++] = pos;
        }
}

// ---------------------------------------------------------------- camera
// base/camera.hpp:23-64 and :108-120 restated in float as glm evaluates
// them (perspective RH, depth 0..1, [1][1] negated); inverse by cofactors.
static V3 cross3(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static void rot_axis(float ang, V3* u, V3* v, V3* n) {
    float s = std::sin(ang), c = std::cos(ang);
    V3 t = (*v) * c + cross3(*u, *v) * s;
    *v = normalize3(t);
    *n = normalize3(cross3(*u, *v));
}

extern "C" void orc_camera_screen_to_world(const float pos[3], const float rot[3], float fov, float aspect, float zn, float zf,
                                float out[16]) {
    const float d2r = 3.14159265358979323846f / 180.0f;
    V3 u = v3(1, 0, 0), v = v3(0, 1, 0), n = v3(0, 0, 1);
    if (rot[1] * d2r != 0.0f) rot_axis(rot[1] * d2r, &v, &n, &u);
    if (rot[0] * d2r != 0.0f) rot_axis(rot[0] * d2r, &u, &v, &n);
    if (rot[2] * d2r != 0.0f) rot_axis(rot[2] * d2r, &n, &u, &v);
    float V[4][4] = {{u.x, v.x, n.x, 0}, {u.y, v.y, n.y, 0}, {u.z, v.z, n.z, 0}, {0, 0, 0, 1}};  // [col][row]
    // translate(M, -p): column 3 = M0*-px + M1*-py + M2*-pz + M3
    for (int r = 0; r < 4; ++r) V[3][r] = V[0][r] * -pos[0] + V[1][r] * -pos[1] + V[2][r] * -pos[2] + V[3][r];
    float th = std::tan(fov * d2r / 2.0f);
    float P[4][4] = {{0}};
    P[0][0] = 1.0f / (aspect * th);
    P[1][1] = 1.0f / th;
    P[2][2] = zf / (zn - zf);
    P[2][3] = -1.0f;
    P[3][2] = -(zf * zn) / (zf - zn);
    P[1][1] *= -1.0f;
    float M[4][4];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) M[c][r] = P[0][r] * V[c][0] + P[1][r] * V[c][1] + P[2][r] * V[c][2] + P[3][r] * V[c][3];
    // Inverse via the adjugate (row-major copy a[r][c]).
    double a[16], inv[16];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) a[r * 4 + c] = M[c][r];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = (float)(inv[r * 4 + c] / det);
}

// --------------------------------------------------------- raygenPrimary
// raygenPrimary.comp:11-26 and :57-84.
static float halton(int i, int base) {
    float r = 0.0f;
    float f = 1.0f / (float)base;
    int j = i;
    while (j > 0) {
        r += f * (float)(j % base);
        j /= base;
        f /= (float)base;
    }
    return r;
}

static void raygen_primary_n(const float m[16], const int32_t* i2p, ORay* rays, const float o[3], int sample_index,
                             int w, int h, float max_dist, long long n) {
    for (long long task = 0; task < n; ++task) {
        int pixel = i2p[task];
        int sx = pixel % w, sy = pixel / w;
        float hx = halton(sample_index, 2), hy = halton(sample_index, 3);
        float x = (float)sx + hx;
        float y = (float)sy + hy;
        float ns[4] = {2.0f * x / (float)w - 1.0f, 2.0f * y / (float)h - 1.0f, 0.0f, 1.0f};
        float wp[4];
        for (int r = 0; r < 4; ++r) wp[r] = m[0 + r] * ns[0] + m[4 + r] * ns[1] + m[8 + r] * ns[2] + m[12 + r] * ns[3];
        V3 world = v3(wp[0] / wp[3], wp[1] / wp[3], wp[2] / wp[3]);
        V3 org = v3(o[0], o[1], o[2]);
        V3 d = normalize3(world - org);
        rays[task] = ORay{o[0], o[1], o[2], 0.0f, d.x, d.y, d.z, max_dist};
    }
}

extern "C" void orc_raygen_primary(const float m[16], const int32_t* i2p, ORay* rays, const float o[3], int sample_index, int w,
                        int h, float max_dist) {
    raygen_primary_n(m, i2p, rays, o, sample_index, w, h, max_dist, (long long)w * h);
}

// ---------------------------------------------------------------- Morton
// computeMortonCodesAila32.comp:39-88.
static void morton_point(const ORay& r, const float* smin, const float* ssize, V3& a, V3& b) {
    V3 q = (v3(r.ox, r.oy, r.oz) - v3(smin[0], smin[1], smin[2])) / v3(ssize[0], ssize[1], ssize[2]);
    a = v3(clamp01(q.x), clamp01(q.y), clamp01(q.z));
    V3 nd = normalize3(v3(r.dx, r.dy, r.dz));
    b = (nd + v3(1.0f, 1.0f, 1.0f)) * 0.5f;
}

static uint32_t aila32_key(V3 a, V3 b) {
    uint32_t iax = (uint32_t)(a.x * 127.0f), iay = (uint32_t)(a.y * 127.0f), iaz = (uint32_t)(a.z * 127.0f);
    uint32_t ibx = (uint32_t)(b.x * 15.0f), iby = (uint32_t)(b.y * 15.0f), ibz = (uint32_t)(b.z * 15.0f);
    uint32_t m = 0;
    m |= ((iax >> 6) & 1) << 31; m |= ((iay >> 6) & 1) << 30; m |= ((iaz >> 6) & 1) << 29;
    m |= ((iax >> 5) & 1) << 28; m |= ((iay >> 5) & 1) << 27; m |= ((iaz >> 5) & 1) << 26;
    m |= ((iax >> 4) & 1) << 25; m |= ((iay >> 4) & 1) << 24; m |= ((iaz >> 4) & 1) << 23;
    m |= ((iax >> 3) & 1) << 22; m |= ((iay >> 3) & 1) << 21; m |= ((iaz >> 3) & 1) << 20;
    m |= ((ibx >> 3) & 1) << 19; m |= ((iby >> 3) & 1) << 18; m |= ((ibz >> 3) & 1) << 17;
    m |= ((iax >> 2) & 1) << 16; m |= ((iay >> 2) & 1) << 15; m |= ((iaz >> 2) & 1) << 14;
    m |= ((ibx >> 2) & 1) << 13; m |= ((iby >> 2) & 1) << 12; m |= ((ibz >> 2) & 1) << 11;
    m |= ((iax >> 1) & 1) << 10; m |= ((iay >> 1) & 1) << 9;  m |= ((iaz >> 1) & 1) << 8;
    m |= ((ibx >> 1) & 1) << 7;  m |= ((iby >> 1) & 1) << 6;  m |= ((ibz >> 1) & 1) << 5;
    m |= ((iax >> 0) & 1) << 4;  m |= ((iay >> 0) & 1) << 3;  m |= ((iaz >> 0) & 1) << 2;
    m |= ((ibx >> 0) & 1) << 1;  m |= ((iby >> 0) & 1) << 0;
    return m;
}

// 6-D interleave by definition: level l holds (ox oy oz dx dy dz) at bits
// 6l+5 .. 6l; origin bits above the direction's width go to the top level's
// slots 6L+2 .. 6L (x, y, z).
static uint64_t key6d(uint32_t o[3], uint32_t d[3], int obits, int dbits) {
    uint64_t k = 0;
    for (int l = 0; l < dbits; ++l) {
        for (int a = 0; a < 3; ++a) k |= (uint64_t)((o[a] >> l) & 1u) << (6 * l + 5 - a);
        for (int a = 0; a < 3; ++a) k |= (uint64_t)((d[a] >> l) & 1u) << (6 * l + 2 - a);
    }
    for (int l = dbits; l < obits; ++l)
        for (int a = 0; a < 3; ++a) k |= (uint64_t)((o[a] >> l) & 1u) << (6 * l + 2 - a);
    return k;
}

extern "C" void orc_morton(const ORay* rays, uint32_t n, const float smin[3], const float ssize[3], int kind, void* keys,
                uint32_t* indices) {
    for (uint32_t i = 0; i < n; ++i) {
        V3 a, b;
        morton_point(rays[i], smin, ssize, a, b);
        if (kind == 0) {
            ((uint32_t*)keys)[i] = aila32_key(a, b);
        } else {
            float os = kind == 1 ? 255.0f : 2047.0f, ds = kind == 1 ? 255.0f : 1023.0f;
            uint32_t o[3] = {(uint32_t)(a.x * os), (uint32_t)(a.y * os), (uint32_t)(a.z * os)};
            uint32_t d[3] = {(uint32_t)(b.x * ds), (uint32_t)(b.y * ds), (uint32_t)(b.z * ds)};
            ((uint64_t*)keys)[i] = kind == 1 ? key6d(o, d, 8, 8) : key6d(o, d, 11, 10);
        }
        indices[i] = i;
    }
}

// ------------------------------------------------------------------ sort
// Stable sort by the low key_bits bits; with indices 0..n-1 as values this
// is the order any stable LSD radix sort produces (vk_radix_sort.h:2598-2755
// sorts 32-bit keys in 4 stable 8-bit passes).
extern "C" void orc_sort_pairs(void* keys, uint32_t* vals, uint32_t n, int key_bits) {
    std::vector<uint32_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0u);
    if (key_bits <= 32) {
        uint32_t* k = (uint32_t*)keys;
        uint32_t mask = key_bits == 32 ? 0xFFFFFFFFu : ((1u << key_bits) - 1u);
        std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return (k[a] & mask) < (k[b] & mask); });
        std::vector<uint32_t> tk(n), tv(n);
        for (uint32_t i = 0; i < n; ++i) {
            tk[i] = k[perm[i]];
            tv[i] = vals[perm[i]];
        }
        std::memcpy(k, tk.data(), n * 4ull);
        std::memcpy(vals, tv.data(), n * 4ull);
    } else {
        uint64_t* k = (uint64_t*)keys;
        uint64_t mask = key_bits == 64 ? ~0ull : ((1ull << key_bits) - 1ull);
        std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return (k[a] & mask) < (k[b] & mask); });
        std::vector<uint64_t> tk(n);
        std::vector<uint32_t> tv(n);
        for (uint32_t i = 0; i < n; ++i) {
            tk[i] = k[perm[i]];
            tv[i] = vals[perm[i]];
        }
        std::memcpy(k, tk.data(), n * 8ull);
        std::memcpy(vals, tv.data(), n * 4ull);
    }
}

// The same stable order by the masked key, by a parallel LSD radix sort with
// 8-bit digits (per-thread digit counts over contiguous chunks, prefix over
// (digit, thread), stable scatter): the multi-threaded CPU baseline of the
// sort stage.  Equal to orc_sort_pairs on every input.
template <class K>
static void lsd_sort_mt(K* keys, uint32_t* vals, uint32_t n, int key_bits) {
    std::vector<K> k2(n);
    std::vector<uint32_t> v2(n);
    K* ka = keys;
    K* kb = k2.data();
    uint32_t* va = vals;
    uint32_t* vb = v2.data();
    const int passes = (key_bits + 7) / 8;
    int T = 1;
#ifdef _OPENMP
    T = std::max(1, omp_get_max_threads());
#endif
    std::vector<uint32_t> counts((size_t)T * 256);
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = 8 * pass;
        const int bits = std::min(8, key_bits - shift);
        const K mask = (K)((1u << bits) - 1u);
        std::fill(counts.begin(), counts.end(), 0u);
#pragma omp parallel num_threads(T)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            uint64_t b = (uint64_t)n * t / T, e = (uint64_t)n * (t + 1) / T;
            uint32_t* c = counts.data() + (size_t)t * 256;
            for (uint64_t i = b; i < e; ++i) ++c[(uint32_t)((ka[i] >> shift) & mask)];
#pragma omp barrier
#pragma omp single
            {
                uint32_t run = 0;
                for (int d = 0; d < 256; ++d)
                    for (int tt = 0; tt < T; ++tt) {
                        uint32_t x = counts[(size_t)tt * 256 + d];
                        counts[(size_t)tt * 256 + d] = run;
                        run += x;
                    }
            }
            for (uint64_t i = b; i < e; ++i) {
                uint32_t dst = c[(uint32_t)((ka[i] >> shift) & mask)]++;
                kb[dst] = ka[i];
                vb[dst] = va[i];
            }
        }
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys) {
        std::memcpy(keys, ka, (size_t)n * sizeof(K));
        std::memcpy(vals, va, (size_t)n * 4);
    }
}

extern "C" void orc_sort_pairs_mt(void* keys, uint32_t* vals, uint32_t n, int key_bits) {
    if (key_bits <= 32)
        lsd_sort_mt((uint32_t*)keys, vals, n, key_bits);
    else
        lsd_sort_mt((uint64_t*)keys, vals, n, key_bits);
}

// --------------------------------------------------------------- reorder
// reorderRays.comp:37-45.
extern "C" void orc_reorder(const uint32_t* idx, const ORay* in_rays, ORay* out_rays, const int32_t* in_s2i, int32_t* out_s2i,
                 int32_t* out_i2s, uint32_t n) {
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        int32_t old = (int32_t)idx[i];
        int32_t index = in_s2i[old];
        out_rays[i] = in_rays[old];
        out_s2i[i] = index;
        out_i2s[index] = (int32_t)i;
    }
}

// The same gather for records of any width (the 48-byte wide-record layout
// of the sort/reorder microbenchmark); slot maps optional (in_s2i null).
extern "C" void orc_reorder_records(const uint32_t* idx, const uint8_t* in_rec, uint8_t* out_rec, uint32_t record_bytes,
                                    const int32_t* in_s2i, int32_t* out_s2i, int32_t* out_i2s, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t old = idx[i];
        std::memcpy(out_rec + (size_t)i * record_bytes, in_rec + (size_t)old * record_bytes, record_bytes);
        if (in_s2i) {
            int32_t index = in_s2i[old];
            out_s2i[i] = index;
            out_i2s[index] = (int32_t)i;
        }
    }
}

// ---------------------------------------------------------- raygenShadow
// raygenShadow.comp:10-44 and :82-136.
static void jenkins(uint32_t& a, uint32_t& b, uint32_t& c) {
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

extern "C" void orc_sobol2d(uint32_t i, float* x, float* y) {
    uint32_t r1 = 0, r2 = 0;
    for (uint32_t v1 = 1u << 31, v2 = 3u << 30; i > 0u; i >>= 1) {
        if ((i & 1u) == 1) {
            r1 ^= v1;
            r2 ^= v2 << 1;
        }
        v1 |= v1 >> 1;
        v2 ^= v2 >> 1;
    }
    *x = (float)r1 / 4294967296.0f;
    *y = (float)r2 / 4294967296.0f;
}

extern "C" void orc_raygen_shadow(const uint32_t* seeds, const ORay* in_rays, const OHit* in_res, ORay* out_rays, int32_t* s2i,
                       int32_t* i2s, const float light[3], float radius, int bb, int bs, int S) {
    const float EPS = 1.0e-5f;
    for (int task = 0; task < bs; ++task) {
        uint32_t seed = seeds[task];
        const ORay& ir = in_rays[bb + task];
        const OHit& res = in_res[bb + task];
        uint32_t ha = seed + (uint32_t)task, hb = 0x9e3779b9u, hc = 0x9e3779b9u;
        jenkins(ha, hb, hc);
        jenkins(ha, hb, hc);
        const float s32 = std::ldexp(1.0f, -32);
        V3 offset = v3((float)ha * s32, (float)hb * s32, (float)hc * s32);
        int tri = res.prim;
        int ray_index = S * task;
        V3 origin = v3(ir.ox, ir.oy, ir.oz) + v3(ir.dx, ir.dy, ir.dz) * std::fmax(res.t - EPS, 0.0f);
        if (tri == -1) origin = v3(0, 0, 0);
        for (int i = 0; i < S; ++i) {
            float sx, sy;
            orc_sobol2d((uint32_t)i, &sx, &sy);
            V3 p = v3(sx, sy, ((float)i + 0.5f) / (float)S);
            p = p + offset;
            if (p.x >= 1.0f) p.x -= 1.0f;
            if (p.y >= 1.0f) p.y -= 1.0f;
            if (p.z >= 1.0f) p.z -= 1.0f;
            p = v3(2.0f * p.x - 1.0f, 2.0f * p.y - 1.0f, 2.0f * p.z - 1.0f);
            V3 target = v3(light[0], light[1], light[2]) + p * radius;
            V3 dir = target - origin;
            V3 nd = tri == -1 ? v3(1, 0, 0) : normalize3(dir);
            float tmax = tri == -1 ? -1.0f : len3(dir);
            out_rays[ray_index] = ORay{origin.x, origin.y, origin.z, EPS, nd.x, nd.y, nd.z, tmax};
            s2i[ray_index] = ray_index;
            i2s[ray_index] = ray_index;
            ++ray_index;
        }
    }
}

// --------------------------------------------------------- unpackTriangle
// geometrytypes.glsl:18-47 (normal only; uv is not used by any stage).
static void unpack_unorm(uint32_t p, float* u, float* v) {
    *u = (float)(p & 0xFFFFu) / 65535.0f;
    *v = (float)(p >> 16) / 65535.0f;
}
static V3 unpack_normal(const OGeom* geoms, int geom, int prim, uint32_t bary) {
    const uint32_t* idx = (const uint32_t*)(uintptr_t)geoms[geom].index_addr;
    const float* vtx = (const float*)(uintptr_t)geoms[geom].vertex_addr;
    float bu, bv;
    unpack_unorm(bary, &bu, &bv);
    float c[3] = {1.0f - bu - bv, bu, bv};
    V3 nsum = v3(0, 0, 0);
    for (int i = 0; i < 3; ++i) {
        size_t off = (size_t)idx[(uint32_t)prim * 3u + i] * 24;  // 6 vec4 per vertex
        V3 ni = v3(vtx[off + 3], vtx[off + 4], vtx[off + 5]);
        nsum = (i == 0) ? ni * c[i] : nsum + ni * c[i];
    }
    return normalize3(nsum);
}

// ------------------------------------------------------------ raygenPath
// raygenPath.comp:16-49 and :95-167; sin/cos of 2*pi*r by the quarter-turn
// reduction plus Taylor series (the shader's float sin/cos are
// implementation-defined; this evaluation is fixed on every platform).
static uint32_t lcg(uint32_t& seed) {
    seed = 1103515245u * seed + 12345u;
    return seed & 0x00FFFFFFu;
}
static float randf(uint32_t& seed) { return (float)lcg(seed) / (float)0x01000000; }

extern "C" void orc_sincos_2pi(float r, float* s, float* c) {
    float q4 = r * 4.0f;
    float q = std::rint(q4);
    float f = q4 - q;
    float x = f * 1.57079632679489662f;
    float x2 = x * x;
    float ps = 1.0f - x2 * (1.0f / 72.0f);
    ps = 1.0f - (x2 * (1.0f / 42.0f)) * ps;
    ps = 1.0f - (x2 * (1.0f / 20.0f)) * ps;
    ps = 1.0f - (x2 * (1.0f / 6.0f)) * ps;
    float sx = x * ps;
    float pc = 1.0f - x2 * (1.0f / 90.0f);
    pc = 1.0f - (x2 * (1.0f / 56.0f)) * pc;
    pc = 1.0f - (x2 * (1.0f / 30.0f)) * pc;
    pc = 1.0f - (x2 * (1.0f / 12.0f)) * pc;
    float cx = 1.0f - (x2 * 0.5f) * pc;
    switch (((int)q) & 3) {
        case 0: *s = sx; *c = cx; break;
        case 1: *s = cx; *c = -sx; break;
        case 2: *s = -sx; *c = -cx; break;
        default: *s = -cx; *c = sx; break;
    }
}

static V3 cosine_dir(float r0, float r1, V3 n) {
    float sn, cs;
    orc_sincos_2pi(r1, &sn, &cs);
    float radius = std::sqrt(r0);
    float x = radius * sn, z = radius * cs, y = std::sqrt(1.0f - r0);
    float s = (n.z >= 0.0f) ? 1.0f : -1.0f;
    float a = -1.0f / (s + n.z);
    float b = n.x * n.y * a;
    V3 u = v3(1.0f + s * n.x * n.x * a, s * b, -(s * n.x));
    V3 w = v3(b, s + n.y * n.y * a, -n.y);
    return u * x + w * z + n * y;
}

// Compaction keeps input order (the reference's subgroup ballot +
// atomicAdd order is nondeterministic).  Returns the number of output rays.
extern "C" uint32_t orc_raygen_path(uint32_t* seeds, const OGeom* geoms, const ORay* in_rays, ORay* out_rays,
                         const int32_t* in_i2p, int32_t* out_i2p, const OHit* in_res, float* decreases, uint32_t n,
                         float albedo) {
    uint32_t count = 0;
    for (uint32_t task = 0; task < n; ++task) {
        int pixel = in_i2p[task];
        uint32_t seed = seeds[task];
        const ORay& ir = in_rays[task];
        const OHit& res = in_res[task];
        if (res.prim < 0) continue;
        V3 dir = v3(ir.dx, ir.dy, ir.dz);
        V3 nrm = unpack_normal(geoms, res.geom, res.prim, res.bary);
        V3 ff = faceforward3(nrm, dir, nrm);
        float r0 = randf(seed);
        float r1 = randf(seed);
        V3 hit = v3(ir.ox, ir.oy, ir.oz) + dir * res.t;
        const float EPS = 1.0e-4f;
        V3 nd = cosine_dir(r0, r1, ff);
        V3 org = hit + nd * EPS;
        out_rays[count] = ORay{org.x, org.y, org.z, EPS, nd.x, nd.y, nd.z, 3.402823466e+38f};
        out_i2p[count] = pixel;
        float* dc = decreases + 4 * (size_t)pixel;
        dc[0] = dc[0] * albedo;
        dc[1] = dc[1] * albedo;
        dc[2] = dc[2] * albedo;
        dc[3] = dc[3] * 1.0f;
        seeds[task] = seed;
        ++count;
    }
    return count;
}

// ----------------------------------------------------- reconstructSmooth
// reconstructSmooth.comp:44-94.
extern "C" void orc_reconstruct_smooth(const ORay* rays, const OHit* res, const int32_t* i2p, float* pixels,
                            const float* decreases, const OGeom* geoms, const float light[3], const float bg[3],
                            uint32_t n, int spp) {
    for (uint32_t task = 0; task < n; ++task) {
        int pixel = i2p[task];
        float* px = pixels + 4 * (size_t)pixel;
        const float* dc = decreases + 4 * (size_t)pixel;
        V3 color = v3(px[0], px[1], px[2]);
        V3 dec = v3(dc[0], dc[1], dc[2]);
        const OHit& r = res[task];
        if (r.prim == -1) {
            color = color + (dec * v3(bg[0], bg[1], bg[2])) / (float)spp;
        } else {
            const ORay& ray = rays[task];
            V3 dir = v3(ray.dx, ray.dy, ray.dz);
            V3 nrm = unpack_normal(geoms, r.geom, r.prim, r.bary);
            V3 L = normalize3(v3(light[0], light[1], light[2]) - (v3(ray.ox, ray.oy, ray.oz) + dir * r.t));
            V3 ff = faceforward3(nrm, dir, nrm);
            float ndl = dot3(ff, L);
            float alpha = std::fmax(ndl, 0.1f);
            color = color + (dec * alpha) / (float)spp;
        }
        px[0] = color.x;
        px[1] = color.y;
        px[2] = color.z;
        px[3] = 1.0f;
    }
}

// ----------------------------------------------------- reconstructShadow
// reconstructShadow.comp:39-59.
extern "C" void orc_reconstruct_shadow(const OHit* res, const int32_t* i2p, const int32_t* i2s, const float* in_pixels,
                            float* out_pixels, int bb, int bs, int S, int replace) {
    for (int task = 0; task < bs; ++task) {
        int pixel = i2p[bb + task];
        const float* ip = in_pixels + 4 * (size_t)pixel;
        float shadow = 0.0f;
        for (int i = 0; i < S; ++i)
            if (res[i2s[task * S + i]].prim == -1) shadow += 1.0f;
        shadow /= (float)S;
        float c[4] = {ip[0] * shadow, ip[1] * shadow, ip[2] * shadow, 1.0f};
        float* op = out_pixels + 4 * (size_t)pixel;
        for (int k = 0; k < 4; ++k) op[k] = replace ? c[k] : op[k] + c[k];
    }
}

// countRayHits.comp:33-49.
extern "C" uint32_t orc_count_hits(const OHit* res, uint32_t n) {
    uint32_t c = 0;
    for (uint32_t i = 0; i < n; ++i) c += res[i].prim >= 0 ? 1u : 0u;
    return c;
}

// ----------------------------------------------------- interpolateColors
// interpolateColors.comp:10-57 (column-major mat3 products) and :78-97.
static V3 reinhard(V3 c, float key, float white) {
    const float avg = 0.5f;
    float X = 0.5141364f * c.x + 0.265068f * c.y + 0.0241188f * c.z;
    float Y = 0.3238786f * c.x + 0.67023428f * c.y + 0.1228178f * c.z;
    float Z = 0.16036376f * c.x + 0.06409157f * c.y + 0.84442666f * c.z;
    float Yl = Y, x = X / (X + Y + Z), y = Y / (X + Y + Z);
    float Lp = Yl * key / avg;
    Yl = (Lp * (1.0f + Lp / (white * white))) / (1.0f + Lp);
    float X2 = Yl * x / y, Y2 = Yl, Z2 = Yl * (1.0f - x - y) / y;
    return v3(2.5651f * X2 + -1.0217f * Y2 + 0.0753f * Z2, -1.1665f * X2 + 1.9777f * Y2 + -0.2543f * Z2,
              -0.3986f * X2 + 0.0439f * Y2 + 1.1892f * Z2);
}

extern "C" void orc_interpolate_colors(float* frame_pixels, float* pixels, uint32_t n, int frame_index, float key, float white) {
    for (uint32_t i = 0; i < n; ++i) {
        float* fp = frame_pixels + 4 * (size_t)i;
        float* pp = pixels + 4 * (size_t)i;
        if (frame_index > 1) {
            V3 c0 = v3(pp[0], pp[1], pp[2]), c1 = v3(fp[0], fp[1], fp[2]);
            float a = 1.0f / (float)frame_index;
            float b = a * ((float)frame_index - 1.0f);
            V3 c = c1 * a + c0 * b;
            pp[0] = c.x; pp[1] = c.y; pp[2] = c.z; pp[3] = 1.0f;
            V3 t = reinhard(c, key, white);
            fp[0] = t.x; fp[1] = t.y; fp[2] = t.z; fp[3] = 1.0f;
        } else {
            for (int k = 0; k < 4; ++k) pp[k] = fp[k];
            V3 t = reinhard(v3(fp[0], fp[1], fp[2]), key, white);
            fp[0] = t.x; fp[1] = t.y; fp[2] = t.z; fp[3] = 1.0f;
        }
    }
}

// The same running mean kept in double (FP64 per-pixel accumulation over
// frames): accum holds 4 doubles per pixel; a = 1/frame and
// b = a * (frame - 1) in double; pixels gets the mean rounded to float (w
// as the shader writes it) and the tone map (float) reads that rounding.
extern "C" void orc_interpolate_colors_fp64(float* frame_pixels, float* pixels, double* accum, uint32_t n,
                                            int frame_index, float key, float white) {
    for (uint32_t i = 0; i < n; ++i) {
        float* fp = frame_pixels + 4 * (size_t)i;
        float* pp = pixels + 4 * (size_t)i;
        double* m = accum + 4 * (size_t)i;
        if (frame_index > 1) {
            double a = 1.0 / (double)frame_index;
            double b = a * ((double)frame_index - 1.0);
            for (int k = 0; k < 3; ++k) m[k] = a * (double)fp[k] + b * m[k];
        } else {
            for (int k = 0; k < 3; ++k) m[k] = (double)fp[k];
        }
        m[3] = 1.0;
        V3 c = v3((float)m[0], (float)m[1], (float)m[2]);
        pp[3] = frame_index > 1 ? 1.0f : fp[3];
        pp[0] = c.x; pp[1] = c.y; pp[2] = c.z;
        V3 t = reinhard(c, key, white);
        fp[0] = t.x; fp[1] = t.y; fp[2] = t.z; fp[3] = 1.0f;
    }
}

// ------------------------------------------------- FP32 BVH2 traversal
// CPU traversal of the 64-byte-node binary BVH (the plain form's format):
// watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013) in float,
// closest hit = smallest t, ties to the smaller global triangle index;
// trace.comp:36-83 semantics (miss = {-1,-1,-1,0}, any-hit for shadows,
// indirect index).  A ray with tmax < tmin misses.
struct TriRec {
    float v0[3];
    int32_t prim;
    float v1[3];
    int32_t geom;
    float v2[3];
    uint32_t global;
};
struct Node2 {
    float f[12];
    int32_t link[4];
};

struct RaySetup {
    float o[3], d[3], inv[3], oinv[3], tmin;
    int kx, ky, kz;
    float sx, sy, sz;
};

static float safe_inv(float d) {
    const float eps = 1e-20f;
    float a = std::fabs(d) > eps ? d : std::copysign(eps, d);
    return 1.0f / a;
}

static RaySetup setup(const ORay& r) {
    RaySetup s;
    s.o[0] = r.ox; s.o[1] = r.oy; s.o[2] = r.oz;
    s.d[0] = r.dx; s.d[1] = r.dy; s.d[2] = r.dz;
    s.tmin = r.tmin;
    for (int k = 0; k < 3; ++k) {
        s.inv[k] = safe_inv(s.d[k]);
        s.oinv[k] = s.o[k] * s.inv[k];
    }
    float ax = std::fabs(r.dx), ay = std::fabs(r.dy), az = std::fabs(r.dz);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (s.d[kz] < 0.0f) std::swap(kx, ky);
    s.kx = kx; s.ky = ky; s.kz = kz;
    s.sx = s.d[kx] / s.d[kz];
    s.sy = s.d[ky] / s.d[kz];
    s.sz = 1.0f / s.d[kz];
    return s;
}

struct Best {
    float t;
    uint32_t key;
    int prim, geom;
    float u, v;
};

static bool tri_test(const RaySetup& r, const TriRec& tr, Best& h) {
    float A[3], B[3], C[3];
    for (int k = 0; k < 3; ++k) {
        A[k] = tr.v0[k] - r.o[k];
        B[k] = tr.v1[k] - r.o[k];
        C[k] = tr.v2[k] - r.o[k];
    }
    float Ax = A[r.kx] - r.sx * A[r.kz], Ay = A[r.ky] - r.sy * A[r.kz];
    float Bx = B[r.kx] - r.sx * B[r.kz], By = B[r.ky] - r.sy * B[r.kz];
    float Cx = C[r.kx] - r.sx * C[r.kz], Cy = C[r.ky] - r.sy * C[r.kz];
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float T = U * (r.sz * A[r.kz]) + V * (r.sz * B[r.kz]) + W * (r.sz * C[r.kz]);
    float t = T / det;
    if (!(t >= r.tmin)) return false;
    if (!(t < h.t || (t == h.t && tr.global < h.key))) return false;
    h.t = t;
    h.key = tr.global;
    h.prim = tr.prim;
    h.geom = tr.geom;
    h.u = V / det;
    h.v = W / det;
    return true;
}

static uint32_t pack_unorm(float u, float v) {
    uint32_t a = (uint32_t)std::nearbyint(clamp01(u) * 65535.0f);
    uint32_t b = (uint32_t)std::nearbyint(clamp01(v) * 65535.0f);
    return a | (b << 16);
}

static bool box_hit(const RaySetup& r, const float lo[3], const float hi[3], float tcur, float* tnear) {
    float t0[3], t1[3];
    for (int k = 0; k < 3; ++k) {
        t0[k] = std::fma(lo[k], r.inv[k], -r.oinv[k]);
        t1[k] = std::fma(hi[k], r.inv[k], -r.oinv[k]);
    }
    float tn = std::fmax(std::fmax(std::fmin(t0[0], t1[0]), std::fmin(t0[1], t1[1])), std::fmax(std::fmin(t0[2], t1[2]), r.tmin));
    float tf = std::fmin(std::fmin(std::fmax(t0[0], t1[0]), std::fmax(t0[1], t1[1])), std::fmin(std::fmax(t0[2], t1[2]), tcur));
    *tnear = tn;
    return tn <= tf * 1.0000004f;
}

static void trace_one(const Node2* nodes, const TriRec* tris, const ORay& ray, OHit& out, int closest) {
    Best h{ray.tmax, 0xFFFFFFFFu, -1, -1, 0, 0};
    bool found = false;
    if (!(ray.tmax >= ray.tmin)) {
        out = OHit{-1, -1, -1.0f, 0};
        return;
    }
    RaySetup r = setup(ray);
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        int node = stack[--sp];
        if (node < 0) {
            uint32_t code = ~(uint32_t)node;
            uint32_t first = code >> 3, cnt = (code & 7u) + 1u;
            bool stop = false;
            for (uint32_t k = 0; k < cnt; ++k)
                if (tri_test(r, tris[first + k], h)) {
                    found = true;
                    if (!closest) {
                        stop = true;
                        break;
                    }
                }
            if (stop) break;
            continue;
        }
        const Node2& n = nodes[node];
        float lo0[3] = {n.f[0], n.f[2], n.f[8]}, hi0[3] = {n.f[1], n.f[3], n.f[9]};
        float lo1[3] = {n.f[4], n.f[6], n.f[10]}, hi1[3] = {n.f[5], n.f[7], n.f[11]};
        float t0, t1;
        bool h0 = box_hit(r, lo0, hi0, h.t, &t0), h1 = box_hit(r, lo1, hi1, h.t, &t1);
        if (h0 && h1) {
            if (t1 < t0) {
                stack[sp++] = n.link[0];
                stack[sp++] = n.link[1];
            } else {
                stack[sp++] = n.link[1];
                stack[sp++] = n.link[0];
            }
        } else if (h0) {
            stack[sp++] = n.link[0];
        } else if (h1) {
            stack[sp++] = n.link[1];
        }
        if (sp > 120) break;  // cannot happen for trees of depth <= 64
    }
    if (found) {
        out = OHit{h.prim, h.geom, h.t, pack_unorm(h.u, h.v)};
    } else {
        out = OHit{-1, -1, -1.0f, 0};
    }
}

extern "C" void orc_trace_bvh2(const void* nodes, const void* tris, const ORay* rays, OHit* results, const uint32_t* ray_index,
                    uint32_t n, int closest) {
    const Node2* N = (const Node2*)nodes;
    const TriRec* T = (const TriRec*)tris;
#pragma omp parallel for schedule(dynamic, 1024)
    for (long long i = 0; i < (long long)n; ++i) {
        uint32_t ri = ray_index ? ray_index[i] : (uint32_t)i;
        trace_one(N, T, rays[ri], results[ri], closest);
    }
}

// ----------------------------------------------------- BVH2 build (own)
// A binned-SAH BVH2 in the traversal format above, independent of the
// product's builder, so that a CPU run needs nothing of the product: 16
// centroid bins per axis, leaves of at most 4 triangles (8 when the SAH
// prefers or the centroids coincide), triangle records in leaf order.
// Stored boxes are grown by 2^-22 * P (P: the largest absolute coordinate)
// so that culling stays conservative for rays that start on a surface.
namespace {
struct BuildTri {
    float lo[3], hi[3], c[3];
};
struct Bvh2Builder {
    const float* pos;
    const uint32_t* idx;
    std::vector<BuildTri> bt;
    std::vector<uint32_t> order;
    std::vector<Node2> nodes;
    float grow = 0.0f;

    static float area(const float lo[3], const float hi[3]) {
        float d[3] = {std::max(0.0f, hi[0] - lo[0]), std::max(0.0f, hi[1] - lo[1]), std::max(0.0f, hi[2] - lo[2])};
        return d[0] * d[1] + d[1] * d[2] + d[2] * d[0];
    }
    void box(uint32_t b, uint32_t e, float lo[3], float hi[3], float clo[3], float chi[3]) const {
        for (int k = 0; k < 3; ++k) lo[k] = clo[k] = FLT_MAX, hi[k] = chi[k] = -FLT_MAX;
        for (uint32_t i = b; i < e; ++i) {
            const BuildTri& t = bt[order[i]];
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], t.lo[k]);
                hi[k] = std::max(hi[k], t.hi[k]);
                clo[k] = std::min(clo[k], t.c[k]);
                chi[k] = std::max(chi[k], t.c[k]);
            }
        }
    }
    int32_t leaf(uint32_t b, uint32_t e) const { return (int32_t)~((b << 3) | (e - b - 1)); }
    // Builds order[b, e); returns its link and writes its (grown) box.  The
    // root is always an inner node (traversal starts at node 0).
    int32_t build(uint32_t b, uint32_t e, float out_lo[3], float out_hi[3], bool root = false) {
        float lo[3], hi[3], clo[3], chi[3];
        box(b, e, lo, hi, clo, chi);
        for (int k = 0; k < 3; ++k) {
            out_lo[k] = lo[k] - grow;
            out_hi[k] = hi[k] + grow;
        }
        const uint32_t n = e - b;
        if (n <= 4 && !root) return leaf(b, e);
        const int NB = 16;
        int best_axis = -1, best_split = 0;
        float best_cost = FLT_MAX;
        for (int ax = 0; ax < 3; ++ax) {
            float ext = chi[ax] - clo[ax];
            if (!(ext > 0.0f)) continue;
            float blo[NB][3], bhi[NB][3];
            uint32_t cnt[NB] = {0};
            for (int i = 0; i < NB; ++i)
                for (int k = 0; k < 3; ++k) blo[i][k] = FLT_MAX, bhi[i][k] = -FLT_MAX;
            for (uint32_t i = b; i < e; ++i) {
                const BuildTri& t = bt[order[i]];
                int bin = std::min(NB - 1, (int)((t.c[ax] - clo[ax]) / ext * NB));
                ++cnt[bin];
                for (int k = 0; k < 3; ++k) {
                    blo[bin][k] = std::min(blo[bin][k], t.lo[k]);
                    bhi[bin][k] = std::max(bhi[bin][k], t.hi[k]);
                }
            }
            float rlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            float rarea[NB];
            uint32_t rcnt[NB];
            uint32_t run = 0;
            for (int i = NB - 1; i > 0; --i) {
                run += cnt[i];
                for (int k = 0; k < 3; ++k) {
                    rlo[k] = std::min(rlo[k], blo[i][k]);
                    rhi[k] = std::max(rhi[k], bhi[i][k]);
                }
                rarea[i] = area(rlo, rhi);
                rcnt[i] = run;
            }
            float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            uint32_t lrun = 0;
            for (int i = 0; i < NB - 1; ++i) {
                lrun += cnt[i];
                for (int k = 0; k < 3; ++k) {
                    llo[k] = std::min(llo[k], blo[i][k]);
                    lhi[k] = std::max(lhi[k], bhi[i][k]);
                }
                if (lrun == 0 || rcnt[i + 1] == 0) continue;
                float cost = area(llo, lhi) * lrun + rarea[i + 1] * rcnt[i + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = ax;
                    best_split = i + 1;
                }
            }
        }
        uint32_t m;
        if (best_axis < 0) {
            if (n <= 8 && !root) return leaf(b, e);
            m = b + n / 2;  // coincident centroids: split by position in the list
        } else {
            // SAH with a node step and a triangle test of equal cost.
            if (n <= 8 && !root && (float)n * area(lo, hi) <= area(lo, hi) + best_cost) return leaf(b, e);
            float ext = chi[best_axis] - clo[best_axis];
            auto mid = std::partition(order.begin() + b, order.begin() + e, [&](uint32_t t) {
                int bin = std::min(NB - 1, (int)((bt[t].c[best_axis] - clo[best_axis]) / ext * NB));
                return bin < best_split;
            });
            m = (uint32_t)(mid - order.begin());
            if (m == b || m == e) m = b + n / 2;
        }
        if (n == 1) m = e;  // a one-triangle scene: both children are that leaf
        int32_t id = (int32_t)nodes.size();
        nodes.push_back(Node2{});
        float l0[3], h0[3], l1[3], h1[3];
        int32_t a = (m == e) ? leaf(b, e) : build(b, m, l0, h0);
        int32_t c = (m == e) ? a : build(m, e, l1, h1);
        if (m == e) {
            for (int k = 0; k < 3; ++k) l0[k] = l1[k] = out_lo[k], h0[k] = h1[k] = out_hi[k];
        }
        Node2& nd = nodes[id];
        nd.f[0] = l0[0]; nd.f[1] = h0[0]; nd.f[2] = l0[1]; nd.f[3] = h0[1];
        nd.f[4] = l1[0]; nd.f[5] = h1[0]; nd.f[6] = l1[1]; nd.f[7] = h1[1];
        nd.f[8] = l0[2]; nd.f[9] = h0[2]; nd.f[10] = l1[2]; nd.f[11] = h1[2];
        nd.link[0] = a;
        nd.link[1] = c;
        nd.link[2] = nd.link[3] = 0;
        return id;
    }
};
}  // namespace

// Builds the BVH2 of ntri triangles (one geometry: primitive id = global
// index = triangle index).  nodes_out holds up to 2 * ntri nodes (64 bytes
// each), tris_out ntri records (48 bytes); returns the node count.
extern "C" uint32_t orc_bvh2_build(const float* pos, const uint32_t* idx, uint32_t ntri, void* nodes_out,
                                   void* tris_out) {
    Bvh2Builder B;
    B.pos = pos;
    B.idx = idx;
    B.bt.resize(ntri);
    B.order.resize(ntri);
    float P = 0.0f;
    for (uint32_t t = 0; t < ntri; ++t) {
        BuildTri& x = B.bt[t];
        for (int k = 0; k < 3; ++k) x.lo[k] = FLT_MAX, x.hi[k] = -FLT_MAX;
        for (int v = 0; v < 3; ++v)
            for (int k = 0; k < 3; ++k) {
                float c = pos[3 * (size_t)idx[3 * (size_t)t + v] + k];
                x.lo[k] = std::min(x.lo[k], c);
                x.hi[k] = std::max(x.hi[k], c);
                P = std::max(P, std::fabs(c));
            }
        for (int k = 0; k < 3; ++k) x.c[k] = 0.5f * (x.lo[k] + x.hi[k]);
        B.order[t] = t;
    }
    B.grow = std::ldexp(P, -22);
    B.nodes.reserve(2 * (size_t)ntri);
    float lo[3], hi[3];
    B.build(0, ntri, lo, hi, true);
    std::memcpy(nodes_out, B.nodes.data(), B.nodes.size() * sizeof(Node2));
    TriRec* T = (TriRec*)tris_out;
    for (uint32_t i = 0; i < ntri; ++i) {
        uint32_t t = B.order[i];
        TriRec r;
        for (int k = 0; k < 3; ++k) {
            r.v0[k] = pos[3 * (size_t)idx[3 * (size_t)t + 0] + k];
            r.v1[k] = pos[3 * (size_t)idx[3 * (size_t)t + 1] + k];
            r.v2[k] = pos[3 * (size_t)idx[3 * (size_t)t + 2] + k];
        }
        r.prim = (int32_t)t;
        r.geom = 0;
        r.global = t;
        T[i] = r;
    }
    return (uint32_t)B.nodes.size();
}

// The seeded synthetic scenes of the benchmark workloads, from the one
// generator the product's wfpt_generate_scene also uses (compiled into this
// library by oracle/build.py), so that a CPU run renders the same triangles
// without loading the product library.  Two calls: sizes first (null
// arrays), then the arrays.
namespace wfpt {
bool generate_scene(int kind, uint64_t seed, uint32_t ntri, std::vector<float>& pos, std::vector<float>& nrm,
                    std::vector<uint32_t>& idx);
}
extern "C" int orc_generate_scene(int kind, uint64_t seed, uint32_t ntri, float* pos, float* nrm, uint32_t* nv,
                                  uint32_t* idx, uint32_t* nt) {
    std::vector<float> p, n;
    std::vector<uint32_t> i;
    if (!wfpt::generate_scene(kind, seed, ntri, p, n, i)) return 0;
    *nv = (uint32_t)(p.size() / 3);
    *nt = (uint32_t)(i.size() / 3);
    if (pos) std::memcpy(pos, p.data(), p.size() * 4);
    if (nrm) std::memcpy(nrm, n.data(), n.size() * 4);
    if (idx) std::memcpy(idx, i.data(), i.size() * 4);
    return 1;
}

// ------------------------------------------------- FP64 traversal oracle
// Independent of the product's BVH: its own median-split BVH over FP64
// triangle boxes and the watertight test evaluated in double.  Reports the
// closest (or any) hit with t in double; geometry index and primitive index
// follow geometry_first (ascending first-triangle offsets).
struct F64Node {
    double lo[3], hi[3];
    int32_t left, right;  // leaf: left = -1 - first, right = count
};

struct F64Scene {
    std::vector<double> v;  // 9 doubles per triangle
    std::vector<uint32_t> order;
    std::vector<F64Node> nodes;
    std::vector<uint32_t> geom_first;
};

static int f64_build(F64Scene& s, uint32_t b, uint32_t e) {
    F64Node nd;
    for (int k = 0; k < 3; ++k) {
        nd.lo[k] = 1e300;
        nd.hi[k] = -1e300;
    }
    for (uint32_t i = b; i < e; ++i) {
        const double* t = &s.v[9 * (size_t)s.order[i]];
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) {
                nd.lo[k] = std::min(nd.lo[k], t[3 * j + k]);
                nd.hi[k] = std::max(nd.hi[k], t[3 * j + k]);
            }
    }
    int id = (int)s.nodes.size();
    s.nodes.push_back(nd);
    if (e - b <= 4) {
        s.nodes[id].left = -1 - (int32_t)b;
        s.nodes[id].right = (int32_t)(e - b);
        return id;
    }
    int ax = 0;
    double ext = -1;
    for (int k = 0; k < 3; ++k)
        if (nd.hi[k] - nd.lo[k] > ext) {
            ext = nd.hi[k] - nd.lo[k];
            ax = k;
        }
    uint32_t m = b + (e - b) / 2;
    std::nth_element(s.order.begin() + b, s.order.begin() + m, s.order.begin() + e, [&](uint32_t x, uint32_t y) {
        const double* a = &s.v[9 * (size_t)x];
        const double* c = &s.v[9 * (size_t)y];
        return a[ax] + a[3 + ax] + a[6 + ax] < c[ax] + c[3 + ax] + c[6 + ax];
    });
    int l = f64_build(s, b, m);
    int r = f64_build(s, m, e);
    s.nodes[id].left = l;
    s.nodes[id].right = r;
    return id;
}

extern "C" void* orc_fp64_scene_create(const float* pos, const uint32_t* idx, uint32_t ntri, const uint32_t* geom_first,
                            uint32_t ngeom) {
    F64Scene* s = new F64Scene();
    s->v.resize(9 * (size_t)ntri);
    for (uint32_t t = 0; t < ntri; ++t)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) s->v[9 * (size_t)t + 3 * j + k] = (double)pos[3 * (size_t)idx[3 * (size_t)t + j] + k];
    s->order.resize(ntri);
    std::iota(s->order.begin(), s->order.end(), 0u);
    if (geom_first && ngeom > 0) s->geom_first.assign(geom_first, geom_first + ngeom);
    else s->geom_first.assign(1, 0u);
    if (ntri > 0) f64_build(*s, 0, ntri);
    return s;
}

extern "C" void orc_fp64_scene_destroy(void* p) { delete (F64Scene*)p; }

struct Best64 {
    double t;
    int64_t tri;
};

static void f64_tri(const double* o, const double* d, int kx, int ky, int kz, double Sx, double Sy, double Sz,
                    const double* tv, uint32_t tri, double tmin, Best64& h, bool& hit) {
    (void)d;  // the direction enters through the permutation (kx, ky, kz) and the shear (Sx, Sy, Sz)
    double A[3], B[3], C[3];
    for (int k = 0; k < 3; ++k) {
        A[k] = tv[k] - o[k];
        B[k] = tv[3 + k] - o[k];
        C[k] = tv[6 + k] - o[k];
    }
    double Ax = A[kx] - Sx * A[kz], Ay = A[ky] - Sy * A[kz];
    double Bx = B[kx] - Sx * B[kz], By = B[ky] - Sy * B[kz];
    double Cx = C[kx] - Sx * C[kz], Cy = C[ky] - Sy * C[kz];
    double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return;
    double det = U + V + W;
    if (det == 0.0) return;
    double T = U * Sz * A[kz] + V * Sz * B[kz] + W * Sz * C[kz];
    double t = T / det;
    if (!(t >= tmin)) return;
    if (!(t < h.t || (t == h.t && (int64_t)tri < h.tri))) return;
    h.t = t;
    h.tri = tri;
    hit = true;
}

// results: t64[i] (or -1), tri64[i] = global triangle index (or -1).
extern "C" void orc_fp64_trace(const void* scene, const ORay* rays, uint32_t n, int closest, double* t64, int64_t* tri64) {
    const F64Scene& s = *(const F64Scene*)scene;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        const ORay& r = rays[i];
        t64[i] = -1.0;
        tri64[i] = -1;
        if (!(r.tmax >= r.tmin) || s.nodes.empty()) continue;
        double o[3] = {r.ox, r.oy, r.oz}, d[3] = {r.dx, r.dy, r.dz};
        double ad[3] = {std::fabs(d[0]), std::fabs(d[1]), std::fabs(d[2])};
        int kz = (ad[0] > ad[1]) ? (ad[0] > ad[2] ? 0 : 2) : (ad[1] > ad[2] ? 1 : 2);
        int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
        if (d[kz] < 0) std::swap(kx, ky);
        double Sx = d[kx] / d[kz], Sy = d[ky] / d[kz], Sz = 1.0 / d[kz];
        double inv[3];
        for (int k = 0; k < 3; ++k) inv[k] = d[k] != 0.0 ? 1.0 / d[k] : std::copysign(1e300, d[k]);
        Best64 h{(double)r.tmax, INT64_MAX};
        bool hit = false;
        int stack[256];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const F64Node& nd = s.nodes[stack[--sp]];
            double tn = r.tmin, tf = h.t;
            bool ok = true;
            for (int k = 0; k < 3 && ok; ++k) {
                double a = (nd.lo[k] - o[k]) * inv[k], b = (nd.hi[k] - o[k]) * inv[k];
                if (a > b) std::swap(a, b);
                // pad by a relative 1e-12 so that the FP64 box test is conservative
                double pad = 1e-12 * (std::fabs(a) + std::fabs(b)) + 1e-300;
                tn = std::max(tn, a - pad);
                tf = std::min(tf, b + pad);
                ok = tn <= tf;
            }
            if (!ok) continue;
            if (nd.left < 0) {
                uint32_t first = (uint32_t)(-1 - nd.left);
                for (int32_t k = 0; k < nd.right; ++k) {
                    uint32_t tri = s.order[first + k];
                    f64_tri(o, d, kx, ky, kz, Sx, Sy, Sz, &s.v[9 * (size_t)tri], tri, r.tmin, h, hit);
                }
                if (hit && !closest) break;
            } else {
                stack[sp++] = nd.left;
                stack[sp++] = nd.right;
            }
        }
        if (hit) {
            t64[i] = h.t;
            tri64[i] = h.tri;
        }
    }
}

// Every triangle tested, no BVH: the closest hit (or the first hit in
// record order for any-hit) under the same watertight test and tie rule.
// Checks that box culling in the traversal above is conservative.
extern "C" void orc_trace_brute(const void* tris, uint32_t num_tris, const ORay* rays, OHit* results, uint32_t n,
                                int closest) {
    const TriRec* T = (const TriRec*)tris;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)n; ++i) {
        const ORay& ray = rays[i];
        OHit& out = results[i];
        out = OHit{-1, -1, -1.0f, 0};
        if (!(ray.tmax >= ray.tmin)) continue;
        RaySetup r = setup(ray);
        Best h{ray.tmax, 0xFFFFFFFFu, -1, -1, 0, 0};
        bool found = false;
        for (uint32_t k = 0; k < num_tris; ++k)
            if (tri_test(r, T[k], h)) {
                found = true;
                if (!closest) break;
            }
        if (found) out = OHit{h.prim, h.geom, h.t, pack_unorm(h.u, h.v)};
    }
}

// ---------------------------------------------------------- whole frame
// Renderer::render with rayType path (Renderer.cpp:552-654, :175-199): the
// CPU pipeline over the same scene, BVH2 and geometry, used for end-to-end
// parity and as the timed CPU baseline.  Sorting and reordering follow the
// flags; reorder changes which seed a path ray reads (seeds are indexed by
// wavefront slot, raygenPath.comp:101), so it is part of the semantics.
struct OFrameCfg {
    int ray_type, spp, S, depth;
    float radius, key, white, albedo;
    int sort_shadow, reorder_shadow, sort_path, reorder_path, morton_kind;
    int frame_index;
    int path_sort_skip;  // bit b: bounce b+1 traces its path rays unsorted
    int accumulate_fp64;  // the running mean in the caller's double buffer
    int pixel_stride;     // > 1: a sample of the frame, every stride-th slot of the pixel table
};

struct OStats {
    uint64_t primary, shadow, path;
    uint32_t path_per_bounce[8];
    uint32_t hits_per_pass[9];
};

static void trace_sort(const Node2* N, const TriRec* T, std::vector<ORay>& rays, std::vector<ORay>& rays_alt,
                       std::vector<int32_t>& s2i, std::vector<int32_t>& s2i_alt, std::vector<int32_t>& i2s_alt,
                       std::vector<OHit>& res, uint32_t n, bool sort, bool reorder, bool closest, const float* smin,
                       const float* ssize, int mk, bool& swapped) {
    if (!sort) {
        orc_trace_bvh2(N, T, rays.data(), res.data(), nullptr, n, closest);
        return;
    }
    std::vector<uint64_t> keys(n);
    std::vector<uint32_t> idx(n);
    int bits = mk == 0 ? 32 : (mk == 1 ? 48 : 63);
    if (mk == 0) {
        std::vector<uint32_t> k32(n);
        orc_morton(rays.data(), n, smin, ssize, 0, k32.data(), idx.data());
        orc_sort_pairs_mt(k32.data(), idx.data(), n, 32);
    } else {
        orc_morton(rays.data(), n, smin, ssize, mk, keys.data(), idx.data());
        orc_sort_pairs_mt(keys.data(), idx.data(), n, bits);
    }
    if (reorder) {
        orc_reorder(idx.data(), rays.data(), rays_alt.data(), s2i.data(), s2i_alt.data(), i2s_alt.data(), n);
        rays.swap(rays_alt);
        s2i.swap(s2i_alt);
        swapped = true;
        orc_trace_bvh2(N, T, rays.data(), res.data(), nullptr, n, closest);
    } else {
        orc_trace_bvh2(N, T, rays.data(), res.data(), idx.data(), n, closest);
    }
}

extern "C" void orc_render_frame(const void* nodes, const void* tris, const OGeom* geoms, const float smin[3], const float smax[3],
                      const float light[3], const float bg[3], const float s2w[16], const float eye[3], float zfar,
                      int w, int h, const OFrameCfg* cfg, float* pixels, float* frame_pixels, OStats* stats,
                      double* accum) {
    const Node2* N = (const Node2*)nodes;
    const TriRec* T = (const TriRec*)tris;
    const uint32_t npx = (uint32_t)w * (uint32_t)h;
    int S = cfg->S;
    float ssize[3] = {smax[0] - smin[0], smax[1] - smin[1], smax[2] - smin[2]};
    std::vector<int32_t> i2p(npx), p2i(npx);
    orc_pixel_table(w, h, i2p.data(), p2i.data());
    // The wavefront: every slot of the pixel table, or with pixel_stride > 1
    // every stride-th one (a sample of the same frame's rays).
    if (cfg->pixel_stride > 1) {
        size_t k = 0;
        for (size_t i = 0; i < npx; i += (size_t)cfg->pixel_stride) i2p[k++] = i2p[i];
        i2p.resize(k);
    }
    const uint32_t n = (uint32_t)i2p.size();
    std::vector<uint32_t> seeds(n);
    std::vector<float> aux(4 * (size_t)npx), dec(4 * (size_t)npx);
    std::memset(stats, 0, sizeof(*stats));
    std::fill(frame_pixels, frame_pixels + 4 * (size_t)npx, 0.0f);
    if (cfg->frame_index == 1) std::fill(pixels, pixels + 4 * (size_t)npx, 0.0f);
    if (cfg->ray_type != 0) orc_init_seeds(seeds.data(), n, cfg->frame_index);
    std::vector<ORay> prim_rays(n);
    std::vector<OHit> prim_res(n);
    const uint32_t kBatch = 8u * 1024u * 1024u;
    auto shadow_pass = [&](const std::vector<ORay>& in_rays, const std::vector<OHit>& in_res,
                           const std::vector<int32_t>& in_s2i, uint32_t n_in, float* in_px, float* out_px,
                           int pass_slot) {
        uint32_t batch_diff = kBatch / (uint32_t)S;
        uint32_t bb = 0;
        do {
            uint32_t be = std::min(bb + batch_diff, n_in), bs = be - bb;
            uint32_t ns = bs * (uint32_t)S;
            std::vector<ORay> sr(ns), sr_alt(ns);
            std::vector<int32_t> s2i(ns), i2s(ns), s2i_alt(ns), i2s_alt(ns);
            std::vector<OHit> sres(ns);
            orc_raygen_shadow(seeds.data(), in_rays.data(), in_res.data(), sr.data(), s2i.data(), i2s.data(), light,
                              cfg->radius, (int)bb, (int)bs, S);
            bool swapped = false;
            trace_sort(N, T, sr, sr_alt, s2i, s2i_alt, i2s_alt, sres, ns, cfg->sort_shadow != 0,
                       cfg->reorder_shadow != 0, false, smin, ssize, cfg->morton_kind, swapped);
            const std::vector<int32_t>& i2s_cur = swapped ? i2s_alt : i2s;
            orc_reconstruct_shadow(sres.data(), in_s2i.data(), i2s_cur.data(), in_px, out_px, (int)bb, (int)bs, S, 0);
            bb = be;
        } while (bb != n_in);
        uint32_t hits = orc_count_hits(in_res.data(), n_in);
        stats->hits_per_pass[pass_slot] += hits;
        stats->shadow += (uint64_t)S * hits;
    };
    for (int pass = 0; pass < cfg->spp; ++pass) {
        float* target = cfg->ray_type == 0 ? frame_pixels : aux.data();
        if (cfg->ray_type != 0) std::fill(aux.begin(), aux.end(), 0.0f);
        int sample_index = pass + cfg->spp * (cfg->frame_index - 1);
        raygen_primary_n(s2w, i2p.data(), prim_rays.data(), eye, sample_index, w, h, zfar, n);
        orc_trace_bvh2(N, T, prim_rays.data(), prim_res.data(), nullptr, n, 1);
        std::fill(dec.begin(), dec.end(), 1.0f);
        orc_reconstruct_smooth(prim_rays.data(), prim_res.data(), i2p.data(), target, dec.data(), geoms, light, bg, n,
                               cfg->spp);
        stats->primary += n;
        if (cfg->ray_type == 0) continue;
        shadow_pass(prim_rays, prim_res, i2p, n, aux.data(), frame_pixels, 0);
        if (cfg->ray_type != 2) continue;
        std::vector<ORay> in_rays = prim_rays;
        std::vector<OHit> in_res = prim_res;
        std::vector<int32_t> in_s2i = i2p;
        uint32_t n_in = n;
        for (int bounce = 0; bounce < cfg->depth; ++bounce) {
            std::fill(aux.begin(), aux.end(), 0.0f);
            std::vector<ORay> out(n), out_alt(n);
            // index_to_slot of the path rays is indexed by pixel (slot_to_index holds pixels)
            std::vector<int32_t> out_s2i(n), s2i_alt(n), i2s_alt(npx);
            std::vector<OHit> out_res(n);
            uint32_t cnt = orc_raygen_path(seeds.data(), geoms, in_rays.data(), out.data(), in_s2i.data(),
                                           out_s2i.data(), in_res.data(), dec.data(), n_in, cfg->albedo);
            stats->path += cnt;
            stats->path_per_bounce[bounce] += cnt;
            bool swapped = false;
            const bool sort_b = cfg->sort_path != 0 && ((cfg->path_sort_skip >> bounce) & 1) == 0;
            trace_sort(N, T, out, out_alt, out_s2i, s2i_alt, i2s_alt, out_res, cnt, sort_b,
                       sort_b && cfg->reorder_path != 0, true, smin, ssize, cfg->morton_kind, swapped);
            orc_reconstruct_smooth(out.data(), out_res.data(), out_s2i.data(), aux.data(), dec.data(), geoms, light, bg,
                                   cnt, cfg->spp);
            if (cnt == 0) break;
            shadow_pass(out, out_res, out_s2i, cnt, aux.data(), frame_pixels, bounce + 1);
            in_rays.swap(out);
            in_res.swap(out_res);
            in_s2i.swap(out_s2i);
            n_in = cnt;
        }
    }
    if (cfg->accumulate_fp64)
        orc_interpolate_colors_fp64(frame_pixels, pixels, accum, npx, cfg->frame_index, cfg->key, cfg->white);
    else
        orc_interpolate_colors(frame_pixels, pixels, npx, cfg->frame_index, cfg->key, cfg->white);
}
