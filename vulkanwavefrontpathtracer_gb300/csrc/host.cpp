// Host-side helpers behind the C ABI: the pixel table, the camera matrix and
// the seeded synthetic scenes that stand in for the reference's glTF assets.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "host.h"

namespace wfpt {

// PixelTable::recalculate (Ray/PixelTable.cpp:39-93): 8x8 pixel blocks
// visited in Morton order of their block coordinates, the 64 pixels of a
// block bit-swizzled, then the bottom stripe (rows not covered by whole
// blocks) column by column, then the right stripe and corner row by row.
void pixel_table(int width, int height, int32_t* idx_to_pix, int32_t* pix_to_idx) {
    int idx = 0;
    int bheight = height & ~7;
    int bwidth = width & ~7;
    int maxdim = bwidth > bheight ? bwidth : bheight;
    // Highest power of two not above maxdim (the reference's "round up"
    // followed by a halving).
    maxdim |= maxdim >> 1;
    maxdim |= maxdim >> 2;
    maxdim |= maxdim >> 4;
    maxdim |= maxdim >> 8;
    maxdim |= maxdim >> 16;
    maxdim = (maxdim + 1) >> 1;
    int width8 = bwidth >> 3;
    int height8 = bheight >> 3;
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
                int pos = (ty * 8 + iy) * width + (tx * 8 + ix);
                pix_to_idx[pos] = idx;
                idx_to_pix[idx++] = pos;
            }
        }
    }
    for (int px = 0; px < bwidth; px++)
        for (int py = bheight; py < height; py++) {
            int pos = px + py * width;
            pix_to_idx[pos] = idx;
            idx_to_pix[idx++] = pos;
        }
    for (int py = 0; py < height; py++)
        for (int px = bwidth; px < width; px++) {
            int pos = px + py * width;
            pix_to_idx[pos] = idx;
            idx_to_pix[idx++] = pos;
        }
}

// ------------------------------------------------------------------ camera
namespace {
struct V3 {
    float x, y, z;
};
V3 cross(V3 a, V3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
V3 nrm(V3 a) {
    float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return {a.x / l, a.y / l, a.z / l};
}
// camera.hpp:47-64: v = normalize(v cos + (u x v) sin), n = normalize(u x v).
void rotate_axis(float ang, V3* u, V3* v, V3* n) {
    float s = std::sin(ang), c = std::cos(ang);
    V3 uv = cross(*u, *v);
    V3 t{v->x * c + uv.x * s, v->y * c + uv.y * s, v->z * c + uv.z * s};
    *v = nrm(t);
    *n = nrm(cross(*u, *v));
}
bool invert4(const double m[16], double out[16]) {
    // Gauss-Jordan with partial pivoting on a column-major 4x4.
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][c + 4] = (r == c) ? 1.0 : 0.0;
        }
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (a[piv][col] == 0.0) return false;
        if (piv != col)
            for (int c = 0; c < 8; ++c) std::swap(a[piv][c], a[col][c]);
        double inv = 1.0 / a[col][col];
        for (int c = 0; c < 8; ++c) a[col][c] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            double f = a[r][col];
            for (int c = 0; c < 8; ++c) a[r][c] -= f * a[col][c];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = a[r][c + 4];
    return true;
}
}  // namespace

// inverse(P * V): camera.hpp:23-45 (view from Euler angles, applied in the
// order y, x, z; view = translate(transpose(rot), -position)) and :108-120
// (perspective, right-handed, depth 0..1, P[1][1] negated), RayGen.cpp:93.
// V, P and their product are evaluated in float in the camera header's
// operation order, as the reference's glm float matrices are (this file is
// compiled without FMA contraction); the product is inverted in double and
// rounded to float.
bool camera_screen_to_world(const float pos[3], const float rot_deg[3], float fov_deg, float aspect, float znear,
                            float zfar, float out[16]) {
    const float d2r = static_cast<float>(3.14159265358979323846 / 180.0);
    V3 u{1, 0, 0}, v{0, 1, 0}, n{0, 0, 1};
    if (rot_deg[1] * d2r != 0.0f) rotate_axis(rot_deg[1] * d2r, &v, &n, &u);
    if (rot_deg[0] * d2r != 0.0f) rotate_axis(rot_deg[0] * d2r, &u, &v, &n);
    if (rot_deg[2] * d2r != 0.0f) rotate_axis(rot_deg[2] * d2r, &n, &u, &v);
    // transpose(mat4(u, v, n, e3)), column-major V[c][r].
    float V[4][4] = {{u.x, v.x, n.x, 0.0f}, {u.y, v.y, n.y, 0.0f}, {u.z, v.z, n.z, 0.0f}, {0.0f, 0.0f, 0.0f, 1.0f}};
    // translate(M, -p): column 3 = M0 * -px + M1 * -py + M2 * -pz + M3.
    const float mp[3] = {-pos[0], -pos[1], -pos[2]};
    for (int r = 0; r < 4; ++r) V[3][r] = V[0][r] * mp[0] + V[1][r] * mp[1] + V[2][r] * mp[2] + V[3][r];
    float th = std::tan(fov_deg * d2r / 2.0f);
    float P[4][4] = {{0.0f}};
    P[0][0] = 1.0f / (aspect * th);
    P[1][1] = 1.0f / th;
    P[2][2] = zfar / (znear - zfar);
    P[2][3] = -1.0f;
    P[3][2] = -(zfar * znear) / (zfar - znear);
    P[1][1] *= -1.0f;
    double PV[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r)
            PV[c * 4 + r] = P[0][r] * V[c][0] + P[1][r] * V[c][1] + P[2][r] * V[c][2] + P[3][r] * V[c][3];
    double inv[16];
    if (!invert4(PV, inv)) return false;
    for (int i = 0; i < 16; ++i) out[i] = (float)inv[i];
    return true;
}

// ----------------------------------------------------------------- scenes
namespace {

struct Rng {
    std::mt19937_64 g;
    explicit Rng(uint64_t s) : g(s) {}
    double uni() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
    double normal() {
        double u1 = uni(), u2 = uni();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

struct Mesh {
    std::vector<float> pos, nrm;
    std::vector<uint32_t> idx;
    uint32_t add_vertex(double x, double y, double z, double nx, double ny, double nz) {
        uint32_t id = (uint32_t)(pos.size() / 3);
        pos.push_back((float)x); pos.push_back((float)y); pos.push_back((float)z);
        nrm.push_back((float)nx); nrm.push_back((float)ny); nrm.push_back((float)nz);
        return id;
    }
    void tri(uint32_t a, uint32_t b, uint32_t c) {
        idx.push_back(a); idx.push_back(b); idx.push_back(c);
    }
    size_t ntri() const { return idx.size() / 3; }
};

// Random triangle around centre c with lognormal edge scale.
void random_triangle(Mesh& m, Rng& r, double cx, double cy, double cz, double mu, double sigma) {
    double v[3][3];
    for (int i = 0; i < 3; ++i) {
        double L = std::exp(mu + sigma * r.normal());
        double dx = r.normal(), dy = r.normal(), dz = r.normal();
        double l = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (l < 1e-12) { dx = 1; dy = 0; dz = 0; l = 1; }
        v[i][0] = cx + L * dx / l;
        v[i][1] = cy + L * dy / l;
        v[i][2] = cz + L * dz / l;
    }
    double e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
    double e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
    double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    double nl = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (nl < 1e-30) { n[0] = 0; n[1] = 1; n[2] = 0; nl = 1; }
    uint32_t a = m.add_vertex(v[0][0], v[0][1], v[0][2], n[0] / nl, n[1] / nl, n[2] / nl);
    uint32_t b = m.add_vertex(v[1][0], v[1][1], v[1][2], n[0] / nl, n[1] / nl, n[2] / nl);
    uint32_t c = m.add_vertex(v[2][0], v[2][1], v[2][2], n[0] / nl, n[1] / nl, n[2] / nl);
    m.tri(a, b, c);
}

// Planar grid: origin o, edge vectors eu (nu cells) and ev (nv cells),
// normal n; optional displacement along n of amplitude `disp`.
void grid(Mesh& m, const double o[3], const double eu[3], const double ev[3], int nu, int nv, const double n[3],
          Rng* r = nullptr, double disp = 0.0) {
    uint32_t base = (uint32_t)(m.pos.size() / 3);
    for (int j = 0; j <= nv; ++j)
        for (int i = 0; i <= nu; ++i) {
            double s = (double)i / nu, t = (double)j / nv;
            double d = (r && disp > 0) ? (2.0 * r->uni() - 1.0) * disp : 0.0;
            m.add_vertex(o[0] + s * eu[0] + t * ev[0] + d * n[0], o[1] + s * eu[1] + t * ev[1] + d * n[1],
                         o[2] + s * eu[2] + t * ev[2] + d * n[2], n[0], n[1], n[2]);
        }
    for (int j = 0; j < nv; ++j)
        for (int i = 0; i < nu; ++i) {
            uint32_t a = base + j * (nu + 1) + i;
            uint32_t b = a + 1, c = a + (nu + 1), d = c + 1;
            m.tri(a, b, d);
            m.tri(a, d, c);
        }
}

void make_soup(Mesh& m, uint64_t seed, uint32_t n) {
    Rng r(seed);
    for (uint32_t i = 0; i < n; ++i) {
        double cx = r.uni(), cy = r.uni(), cz = r.uni();
        random_triangle(m, r, cx, cy, cz, -4.0, 0.5);
    }
}

// Box room 30 x 12 x 20 (x, y up, z), 5 cells per unit, normals inward;
// 48 cylinders (8 x 6, radius 0.35, 32 segments x 32 stacks = 2048
// triangles each); 50,000 clutter triangles in the room.
void make_courtyard(Mesh& m, uint64_t seed) {
    Rng r(seed);
    const double X = 30, Y = 12, Z = 20;
    const int cpu = 5;
    {
        double o[3] = {0, 0, 0}, eu[3] = {X, 0, 0}, ev[3] = {0, 0, Z}, n[3] = {0, 1, 0};
        grid(m, o, ev, eu, (int)(Z * cpu), (int)(X * cpu), n);  // floor
    }
    {
        double o[3] = {0, Y, 0}, eu[3] = {X, 0, 0}, ev[3] = {0, 0, Z}, n[3] = {0, -1, 0};
        grid(m, o, eu, ev, (int)(X * cpu), (int)(Z * cpu), n);  // ceiling
    }
    {
        double o[3] = {0, 0, 0}, eu[3] = {0, 0, Z}, ev[3] = {0, Y, 0}, n[3] = {1, 0, 0};
        grid(m, o, eu, ev, (int)(Z * cpu), (int)(Y * cpu), n);  // x = 0
    }
    {
        double o[3] = {X, 0, 0}, eu[3] = {0, Y, 0}, ev[3] = {0, 0, Z}, n[3] = {-1, 0, 0};
        grid(m, o, eu, ev, (int)(Y * cpu), (int)(Z * cpu), n);  // x = X
    }
    {
        double o[3] = {0, 0, 0}, eu[3] = {0, Y, 0}, ev[3] = {X, 0, 0}, n[3] = {0, 0, 1};
        grid(m, o, eu, ev, (int)(Y * cpu), (int)(X * cpu), n);  // z = 0
    }
    {
        double o[3] = {0, 0, Z}, eu[3] = {X, 0, 0}, ev[3] = {0, Y, 0}, n[3] = {0, 0, -1};
        grid(m, o, eu, ev, (int)(X * cpu), (int)(Y * cpu), n);  // z = Z
    }
    const int seg = 32, stacks = 32;
    const double rad = 0.35;
    for (int gz = 0; gz < 6; ++gz)
        for (int gx = 0; gx < 8; ++gx) {
            double cx = 3.0 + gx * 24.0 / 7.0, cz = 2.5 + gz * 15.0 / 5.0;
            uint32_t base = (uint32_t)(m.pos.size() / 3);
            for (int j = 0; j <= stacks; ++j)
                for (int i = 0; i < seg; ++i) {
                    double a = 6.283185307179586 * i / seg;
                    double nx = std::cos(a), nz = std::sin(a);
                    m.add_vertex(cx + rad * nx, Y * j / stacks, cz + rad * nz, nx, 0, nz);
                }
            for (int j = 0; j < stacks; ++j)
                for (int i = 0; i < seg; ++i) {
                    uint32_t a = base + j * seg + i, b = base + j * seg + (i + 1) % seg;
                    uint32_t c = a + seg, d = b + seg;
                    m.tri(a, c, d);
                    m.tri(a, d, b);
                }
        }
    for (int i = 0; i < 50000; ++i) {
        double cx = 1 + 28 * r.uni(), cy = 0.5 + 5.5 * r.uni(), cz = 1 + 18 * r.uni();
        random_triangle(m, r, cx, cy, cz, -2.5, 0.5);
    }
}

// City block: G x G boxes (cell 10, footprint 7 x 7, seeded heights 5..40),
// top and four sides each subdivided 9 x 8 quads and displaced by +-2% of
// the footprint along the face normal, on a ground grid of 160 x 160 quads.
// G = 64 gives 3,000,320 triangles.
void make_city(Mesh& m, uint64_t seed, int G) {
    Rng r(seed);
    const double cell = 10.0, foot = 7.0, disp = 0.02 * foot;
    const int a = 9, b = 8;
    {
        double ext = G * cell;
        double o[3] = {0, 0, 0}, eu[3] = {0, 0, ext}, ev[3] = {ext, 0, 0}, n[3] = {0, 1, 0};
        int gq = std::max(1, 160 * G / 64);
        grid(m, o, eu, ev, gq, gq, n);
    }
    for (int gz = 0; gz < G; ++gz)
        for (int gx = 0; gx < G; ++gx) {
            double h = 5.0 + 35.0 * r.uni();
            double x0 = gx * cell + (cell - foot) / 2, z0 = gz * cell + (cell - foot) / 2;
            double x1 = x0 + foot, z1 = z0 + foot;
            {
                double o[3] = {x0, h, z0}, eu[3] = {0, 0, foot}, ev[3] = {foot, 0, 0}, n[3] = {0, 1, 0};
                grid(m, o, eu, ev, a, b, n, &r, disp);
            }
            {
                double o[3] = {x0, 0, z0}, eu[3] = {foot, 0, 0}, ev[3] = {0, h, 0}, n[3] = {0, 0, -1};
                grid(m, o, eu, ev, a, b, n, &r, disp);
            }
            {
                double o[3] = {x1, 0, z1}, eu[3] = {-foot, 0, 0}, ev[3] = {0, h, 0}, n[3] = {0, 0, 1};
                grid(m, o, eu, ev, a, b, n, &r, disp);
            }
            {
                double o[3] = {x0, 0, z1}, eu[3] = {0, 0, -foot}, ev[3] = {0, h, 0}, n[3] = {-1, 0, 0};
                grid(m, o, eu, ev, a, b, n, &r, disp);
            }
            {
                double o[3] = {x1, 0, z0}, eu[3] = {0, 0, foot}, ev[3] = {0, h, 0}, n[3] = {1, 0, 0};
                grid(m, o, eu, ev, a, b, n, &r, disp);
            }
        }
}

}  // namespace

bool generate_scene(int kind, uint64_t seed, uint32_t ntri, std::vector<float>& pos, std::vector<float>& nrm,
                    std::vector<uint32_t>& idx) {
    Mesh m;
    switch (kind) {
        case 0: make_soup(m, seed, ntri); break;
        case 1: make_courtyard(m, seed); break;
        case 2: make_city(m, seed, 64); break;
        case 3: {
            int G = std::max(1, (int)std::lround(std::sqrt((double)ntri / 732.0)));
            make_city(m, seed, G);
            break;
        }
        default: return false;
    }
    pos.swap(m.pos);
    nrm.swap(m.nrm);
    idx.swap(m.idx);
    return true;
}

}  // namespace wfpt
