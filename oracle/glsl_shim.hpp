// GLSL compute-shader semantics in C++, for running the reference's own
// shader sources on the CPU (test infrastructure only: oracle/ref_build.py
// rewrites each .comp file's declarations into the forms below and compiles
// the function bodies unchanged against this header).
//
// Arithmetic model, chosen so that the result is one valid GLSL evaluation
// and comparable bit for bit with the restatement in oracle.cpp:
// - float + - * / and sqrt are IEEE single precision, round to nearest, with
//   no contraction into FMA (the recipe compiles with -ffp-contract=off);
//   GLSL literals without a suffix are float (the recipe adds the suffix).
// - dot() sums its products left to right; length(v) = sqrt(dot(v, v));
//   normalize(v) = v / length(v), component by component (the GLSL
//   specification's definition); matrix * vector sums columns 0..n-1 left
//   to right.
// - min/max/clamp follow the specification's definitions
//   (max(x, y) = x < y ? y : x), faceforward(N, I, Nref) = dot(Nref, I) < 0
//   ? N : -N, unpackUnorm2x16 divides each 16-bit field by 65535.
// - sin/cos/exp2 are the C library's single-precision functions; GLSL leaves
//   their precision to the implementation.
// Invocations run one at a time.  Shaders that use subgroup operations or
// barrier() run each invocation of a workgroup as a fiber (ucontext): an
// invocation that reaches a subgroup operation waits until every invocation
// of its subgroup that has not returned reaches it, then all of them get
// their results; barrier() waits for the whole workgroup.  Subgroups of a
// workgroup, and workgroups, run in index order, so an atomic counter bumped
// once per subgroup hands out offsets in invocation order.
#pragma once

#include <ucontext.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace glsl {

typedef uint32_t uint;

template <int N, int A, int B>
struct Swz2;
template <int N, int A, int B, int C>
struct Swz3;

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};

struct vec4;

struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(float a, vec2 b) : x(a), y(b.x), z(b.y) {}
    vec3(vec2 a, float c) : x(a.x), y(a.y), z(c) {}
    explicit vec3(const vec4& v);
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};

template <int N, int A, int B>
struct Swz2 {
    float e[N];
    operator vec2() const { return vec2(e[A], e[B]); }
};
template <int N, int A, int B, int C>
struct Swz3 {
    float e[N];
    operator vec3() const { return vec3(e[A], e[B], e[C]); }
};

struct vec4 {
    union {
        struct {
            float x, y, z, w;
        };
        Swz2<4, 0, 1> xy;
        Swz2<4, 2, 3> zw;
        Swz3<4, 0, 1, 2> xyz;
    };
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(vec3 a, float d) : x(a.x), y(a.y), z(a.z), w(d) {}
    vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    vec4& operator=(const vec4& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        w = o.w;
        return *this;
    }
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};
static_assert(sizeof(vec2) == 8 && sizeof(vec3) == 12 && sizeof(vec4) == 16, "std430 element sizes");

inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
};

struct uvec3 {
    uint x, y, z;
    uvec3() : x(0), y(0), z(0) {}
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    // GLSL uvec3(vec3): each component converted as uint(float) (truncation).
    explicit uvec3(vec3 v) : x((uint)v.x), y((uint)v.y), z((uint)v.z) {}
};

struct uvec4 {
    uint x, y, z, w;
    uvec4() : x(0), y(0), z(0), w(0) {}
    uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};

// Component-wise operators, written out per type.
#define GLSL_VEC_OPS(V, N)                                                                  \
    inline V operator+(V a, V b) {                                                          \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r[i] = a[i] + b[i];                                     \
        return r;                                                                           \
    }                                                                                       \
    inline V operator-(V a, V b) {                                                          \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r[i] = a[i] - b[i];                                     \
        return r;                                                                           \
    }                                                                                       \
    inline V operator*(V a, V b) {                                                          \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r[i] = a[i] * b[i];                                     \
        return r;                                                                           \
    }                                                                                       \
    inline V operator/(V a, V b) {                                                          \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r[i] = a[i] / b[i];                                     \
        return r;                                                                           \
    }                                                                                       \
    inline V operator+(V a, float s) { return a + V(s); }                                   \
    inline V operator-(V a, float s) { return a - V(s); }                                   \
    inline V operator*(V a, float s) { return a * V(s); }                                   \
    inline V operator/(V a, float s) { return a / V(s); }                                   \
    inline V operator+(float s, V a) { return V(s) + a; }                                   \
    inline V operator-(float s, V a) { return V(s) - a; }                                   \
    inline V operator*(float s, V a) { return V(s) * a; }                                   \
    inline V operator/(float s, V a) { return V(s) / a; }                                   \
    inline V operator-(V a) {                                                               \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r[i] = -a[i];                                           \
        return r;                                                                           \
    }                                                                                       \
    inline V& operator+=(V& a, V b) { return a = a + b; }                                   \
    inline V& operator-=(V& a, V b) { return a = a - b; }                                   \
    inline V& operator*=(V& a, V b) { return a = a * b; }                                   \
    inline V& operator/=(V& a, V b) { return a = a / b; }                                   \
    inline V& operator*=(V& a, float s) { return a = a * s; }                               \
    inline V& operator/=(V& a, float s) { return a = a / s; }                               \
    inline float dot(V a, V b) {                                                            \
        float s = a[0] * b[0];                                                              \
        for (int i = 1; i < N; ++i) s = s + a[i] * b[i];                                    \
        return s;                                                                           \
    }                                                                                       \
    inline float length(V a) { return std::sqrt(dot(a, a)); }                              \
    inline V normalize(V a) { return a / length(a); }                                       \
    inline V faceforward(V n, V i, V nref) { return dot(nref, i) < 0.0f ? n : -n; }         \
    inline V clamp(V a, float lo, float hi) {                                               \
        V r;                                                                                \
        for (int i = 0; i < N; ++i) r[i] = clamp(a[i], lo, hi);                             \
        return r;                                                                           \
    }

inline float max(float x, float y) { return x < y ? y : x; }
inline float min(float x, float y) { return y < x ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float exp2(float x) { return std::exp2(x); }
inline float abs(float x) { return std::fabs(x); }

GLSL_VEC_OPS(vec2, 2)
GLSL_VEC_OPS(vec3, 3)
GLSL_VEC_OPS(vec4, 4)
#undef GLSL_VEC_OPS

// Column-major matrices: c[j] is column j.
struct mat3 {
    vec3 c[3];
    mat3(float a0, float a1, float a2, float a3, float a4, float a5, float a6, float a7, float a8) {
        c[0] = vec3(a0, a1, a2);
        c[1] = vec3(a3, a4, a5);
        c[2] = vec3(a6, a7, a8);
    }
    vec3& operator[](int j) { return c[j]; }
    const vec3& operator[](int j) const { return c[j]; }
};
inline vec3 operator*(const mat3& m, vec3 v) {
    vec3 r;
    for (int i = 0; i < 3; ++i) r[i] = m[0][i] * v[0] + m[1][i] * v[1] + m[2][i] * v[2];
    return r;
}

struct mat4 {
    vec4 c[4];
    mat4() {}
    vec4& operator[](int j) { return c[j]; }
    const vec4& operator[](int j) const { return c[j]; }
};
inline vec4 operator*(const mat4& m, vec4 v) {
    vec4 r;
    for (int i = 0; i < 4; ++i) r[i] = m[0][i] * v[0] + m[1][i] * v[1] + m[2][i] * v[2] + m[3][i] * v[3];
    return r;
}

inline vec2 unpackUnorm2x16(uint p) {
    return vec2((float)(p & 0xffffu) / 65535.0f, (float)(p >> 16) / 65535.0f);
}

inline uint atomicAdd(uint& mem, uint v) {
    uint old = mem;
    mem = old + v;
    return old;
}

// Buffer references (GL_EXT_buffer_reference): a struct built from a
// 64-bit address; the recipe rewrites each block declaration into one of
// these.
#define GLSL_BUFFER_ARRAY(Name, Type, field)                                                   \
    struct Name {                                                                              \
        Type* field;                                                                           \
        explicit Name(uint64_t a) : field(reinterpret_cast<Type*>((uintptr_t)a)) {}            \
    }
#define GLSL_BUFFER_SCALAR(Name, Type, field)                                                  \
    struct Name {                                                                              \
        Type& field;                                                                           \
        explicit Name(uint64_t a) : field(*reinterpret_cast<Type*>((uintptr_t)a)) {}           \
    }

// ------------------------------------------------------------- dispatch
// Built-in variables of the invocation that runs now.
inline uvec3 gl_GlobalInvocationID;
inline uvec3 gl_LocalInvocationID;
inline uvec3 gl_WorkGroupID;
inline uint gl_SubgroupID = 0;
inline uint gl_SubgroupInvocationID = 0;
inline uint gl_NumSubgroups = 1;
inline uint gl_SubgroupSize = 32;

enum Op { OP_NONE = 0, OP_BALLOT, OP_ELECT, OP_BROADCAST_FIRST, OP_ADD, OP_BARRIER };

struct Fiber {
    ucontext_t ctx;
    std::vector<char> stack;
    bool done = false;
    Op op = OP_NONE;
    uint64_t arg = 0;
    uint64_t result = 0;
};

struct Dispatch {
    std::vector<Fiber> fibers;
    ucontext_t sched;
    int cur = 0;
    void (*fn)() = nullptr;
};
inline Dispatch* g_dispatch = nullptr;

[[noreturn]] inline void fail(const char* msg) {
    std::fprintf(stderr, "glsl shim: %s\n", msg);
    std::abort();
}

inline uint64_t rendezvous(Op op, uint64_t arg) {
    Dispatch* d = g_dispatch;
    if (!d) fail("subgroup operation or barrier() outside a fiber dispatch");
    Fiber& me = d->fibers[d->cur];
    me.op = op;
    me.arg = arg;
    swapcontext(&me.ctx, &d->sched);
    return me.result;
}

inline uvec4 subgroupBallot(bool v) {
    uint64_t m = rendezvous(OP_BALLOT, v ? 1 : 0);
    return uvec4((uint)m, (uint)(m >> 32), 0, 0);
}
inline uint subgroupBallotBitCount(uvec4 b) {
    return (uint)(__builtin_popcount(b.x) + __builtin_popcount(b.y) + __builtin_popcount(b.z) +
                  __builtin_popcount(b.w));
}
inline uint subgroupBallotExclusiveBitCount(uvec4 b) {
    uint lane = gl_SubgroupInvocationID, n = 0;
    uint w[4] = {b.x, b.y, b.z, b.w};
    for (uint i = 0; i < 4; ++i) {
        if (lane >= 32 * (i + 1)) {
            n += (uint)__builtin_popcount(w[i]);
        } else {
            uint bits = lane - 32 * i;
            n += bits ? (uint)__builtin_popcount(w[i] & ((bits >= 32) ? 0xffffffffu : ((1u << bits) - 1u))) : 0u;
            break;
        }
    }
    return n;
}
inline bool subgroupElect() { return rendezvous(OP_ELECT, 0) != 0; }
inline uint subgroupBroadcastFirst(uint v) { return (uint)rendezvous(OP_BROADCAST_FIRST, v); }
inline uint subgroupAdd(uint v) { return (uint)rendezvous(OP_ADD, v); }
inline void barrier() { rendezvous(OP_BARRIER, 0); }

inline void fiber_entry() {
    Dispatch* d = g_dispatch;
    d->fn();
    d->fibers[d->cur].done = true;
}

inline void set_builtins(uint group, uint local, uint local_size) {
    gl_WorkGroupID = uvec3(group, 0, 0);
    gl_LocalInvocationID = uvec3(local, 0, 0);
    gl_GlobalInvocationID = uvec3(group * local_size + local, 0, 0);
    gl_SubgroupID = local / gl_SubgroupSize;
    gl_SubgroupInvocationID = local % gl_SubgroupSize;
    gl_NumSubgroups = (local_size + gl_SubgroupSize - 1) / gl_SubgroupSize;
}

// Runs `groups` workgroups of `local_size` invocations of fn.  With
// fibers == false every invocation runs to completion in turn (shaders
// without subgroup operations or barriers).
inline void dispatch(uint groups, uint local_size, void (*fn)(), bool fibers, uint subgroup_size = 32) {
    gl_SubgroupSize = subgroup_size;
    if (!fibers) {
        for (uint g = 0; g < groups; ++g)
            for (uint l = 0; l < local_size; ++l) {
                set_builtins(g, l, local_size);
                fn();
            }
        return;
    }
    Dispatch d;
    d.fn = fn;
    d.fibers.resize(local_size);
    for (Fiber& f : d.fibers) f.stack.resize(128 * 1024);
    Dispatch* saved = g_dispatch;
    g_dispatch = &d;
    const uint nsg = (local_size + subgroup_size - 1) / subgroup_size;
    for (uint g = 0; g < groups; ++g) {
        for (uint l = 0; l < local_size; ++l) {
            Fiber& f = d.fibers[l];
            f.done = false;
            f.op = OP_NONE;
            getcontext(&f.ctx);
            f.ctx.uc_stack.ss_sp = f.stack.data();
            f.ctx.uc_stack.ss_size = f.stack.size();
            f.ctx.uc_link = &d.sched;
            makecontext(&f.ctx, fiber_entry, 0);
        }
        // f.op == OP_NONE and !f.done: runnable.
        for (;;) {
            for (uint sg = 0; sg < nsg; ++sg) {
                const uint l0 = sg * subgroup_size, l1 = std::min(local_size, l0 + subgroup_size);
                for (;;) {
                    for (uint l = l0; l < l1; ++l) {
                        Fiber& f = d.fibers[l];
                        if (f.done || f.op != OP_NONE) continue;
                        d.cur = (int)l;
                        set_builtins(g, l, local_size);
                        swapcontext(&d.sched, &f.ctx);
                    }
                    // Every invocation of the subgroup has returned or waits.
                    Op op = OP_NONE;
                    int first = -1;
                    bool any_barrier = false;
                    for (uint l = l0; l < l1; ++l) {
                        Fiber& f = d.fibers[l];
                        if (f.done) continue;
                        if (f.op == OP_BARRIER) {
                            any_barrier = true;
                            continue;
                        }
                        if (op == OP_NONE) {
                            op = f.op;
                            first = (int)l;
                        } else if (f.op != op) {
                            fail("invocations of one subgroup wait on different subgroup operations");
                        }
                    }
                    if (op == OP_NONE) break;
                    if (any_barrier) fail("a subgroup operation and barrier() reached in one subgroup");
                    uint64_t ballot = 0, sum = 0;
                    for (uint l = l0; l < l1; ++l) {
                        Fiber& f = d.fibers[l];
                        if (f.done) continue;
                        if (f.arg) ballot |= 1ull << (l - l0);
                        sum += f.arg;
                    }
                    for (uint l = l0; l < l1; ++l) {
                        Fiber& f = d.fibers[l];
                        if (f.done) continue;
                        switch (op) {
                            case OP_BALLOT: f.result = ballot; break;
                            case OP_ELECT: f.result = ((int)l == first) ? 1 : 0; break;
                            case OP_BROADCAST_FIRST: f.result = d.fibers[first].arg; break;
                            case OP_ADD: f.result = (uint32_t)sum; break;
                            default: fail("unknown subgroup operation");
                        }
                        f.op = OP_NONE;
                    }
                }
            }
            bool waiting = false, all_done = true;
            for (Fiber& f : d.fibers) {
                if (!f.done) all_done = false;
                if (!f.done && f.op == OP_BARRIER) waiting = true;
            }
            if (all_done) break;
            if (!waiting) fail("workgroup neither finished nor waiting at barrier()");
            for (Fiber& f : d.fibers)
                if (!f.done) f.op = OP_NONE;  // release the barrier
        }
    }
    g_dispatch = saved;
}

inline uint groups_for(uint64_t n, uint local_size) { return (uint)((n + local_size - 1) / local_size); }

}  // namespace glsl
