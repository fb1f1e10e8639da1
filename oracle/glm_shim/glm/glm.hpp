// A small stand-in for the parts of glm that the reference's camera header
// (base/camera.hpp) uses, written from the mathematics (glm itself is an
// empty submodule in the reference).  Test infrastructure only: it lets
// oracle/ref_build.py compile that header unchanged, so that its rotation
// order, view composition and projection set-up are the reference's own.
// Column-major 4x4 matrices (m[c][r]); perspective is the right-handed,
// depth 0..1 projection that GLM_FORCE_DEPTH_ZERO_TO_ONE selects; inverse
// is Gauss-Jordan elimination in double, rounded to float.
#pragma once

#include <cmath>

namespace glm {

struct vec2 {
    float x = 0, y = 0;
    vec2() = default;
    vec2(float a, float b) : x(a), y(b) {}
};

struct vec3 {
    float x = 0, y = 0, z = 0;
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return a * s; }
inline vec3& operator+=(vec3& a, vec3 b) { return a = a + b; }
inline vec3& operator-=(vec3& a, vec3 b) { return a = a - b; }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline vec3 normalize(vec3 a) {
    float l = std::sqrt(dot(a, a));
    return vec3(a.x / l, a.y / l, a.z / l);
}

struct vec4 {
    float x = 0, y = 0, z = 0, w = 0;
    vec4() = default;
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(vec3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};
inline bool operator==(const vec4& a, const vec4& b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }

struct mat4 {
    vec4 c[4];
    mat4() : mat4(1.0f) {}
    explicit mat4(float d) {
        for (int j = 0; j < 4; ++j)
            for (int i = 0; i < 4; ++i) c[j][i] = (i == j) ? d : 0.0f;
    }
    mat4(vec4 a, vec4 b, vec4 d, vec4 e) : c{a, b, d, e} {}
    vec4& operator[](int j) { return c[j]; }
    const vec4& operator[](int j) const { return c[j]; }
};
inline bool operator==(const mat4& a, const mat4& b) {
    return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3];
}
inline bool operator!=(const mat4& a, const mat4& b) { return !(a == b); }
// (A B)[j][r] = sum over k = 0..3, left to right, of A[k][r] * B[j][k].
inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r(0.0f);
    for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 4; ++i) r[j][i] = a[0][i] * b[j][0] + a[1][i] * b[j][1] + a[2][i] * b[j][2] + a[3][i] * b[j][3];
    return r;
}

inline float radians(float deg) { return deg * static_cast<float>(3.14159265358979323846 / 180.0); }

inline mat4 transpose(const mat4& m) {
    mat4 r(0.0f);
    for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 4; ++i) r[j][i] = m[i][j];
    return r;
}

// m * T(v): column 3 becomes m0 v.x + m1 v.y + m2 v.z + m3.
inline mat4 translate(const mat4& m, vec3 v) {
    mat4 r = m;
    for (int i = 0; i < 4; ++i) r[3][i] = m[0][i] * v.x + m[1][i] * v.y + m[2][i] * v.z + m[3][i];
    return r;
}

// Right-handed view space (looking down -z), clip depth 0 at near, 1 at far.
inline mat4 perspective(float fovy, float aspect, float zn, float zf) {
    float t = std::tan(fovy / 2.0f);
    mat4 r(0.0f);
    r[0][0] = 1.0f / (aspect * t);
    r[1][1] = 1.0f / t;
    r[2][2] = zf / (zn - zf);
    r[2][3] = -1.0f;
    r[3][2] = -(zf * zn) / (zf - zn);
    return r;
}

inline mat4 inverse(const mat4& m) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c][r];
            a[r][c + 4] = (r == c) ? 1.0 : 0.0;
        }
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (piv != col)
            for (int k = 0; k < 8; ++k) std::swap(a[col][k], a[piv][k]);
        double p = a[col][col];
        for (int k = 0; k < 8; ++k) a[col][k] /= p;
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            double f = a[r][col];
            for (int k = 0; k < 8; ++k) a[r][k] -= f * a[col][k];
        }
    }
    mat4 out(0.0f);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c][r] = (float)a[r][c + 4];
    return out;
}

}  // namespace glm
