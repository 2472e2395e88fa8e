// Project-written shim under which the reference's Slang compute shaders compile as C++ on the
// CPU (test infrastructure: it builds the reference's own step code as a checker for the oracle).
//
// It supplies the HLSL/Slang vocabulary those shaders use: scalar-layout vectors (float3 is 12
// bytes, as the reference's glm::vec3 buffers), a row-major float4x4 with mul(M, v) = M v, the
// intrinsics (floor, sqrt, pow, length, dot, min, max, abs, any), ConstantBuffer<T>, the
// Interlocked adds (plain adds: the host driver runs the passes that use them in index order on one
// thread, so the counting sort is stable), and group barriers (a kernel with barriers runs its
// group's threads as cooperative fibers that switch at every barrier).
//
// Buffer pointers are bounds-checked views (ref_ptr): an out-of-range access aborts with a
// message instead of reading past the buffer, and so do float -> integer conversions that C++
// leaves undefined. Fixtures are only generated from runs that do neither.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <csetjmp>
#include <setjmp.h>
#include <ucontext.h>

typedef uint32_t uint;

namespace slang_shim {
[[noreturn]] inline void fault(const char* what, long long a = 0, long long b = 0) {
    std::fprintf(stderr, "reference shader run: %s (%lld, %lld)\n", what, a, b);
    std::abort();
}
}  // namespace slang_shim

// ------------------------------------------------------------------ buffers
template <class T>
struct ref_ptr {
    T* p = nullptr;
    size_t n = 0;
    template <class I>
    T& operator[](I i) const {
        if (i < 0 || (size_t)i >= n) slang_shim::fault("buffer index out of range", (long long)i, (long long)n);
        return p[(size_t)i];
    }
};

template <class T>
using ConstantBuffer = T;

// ------------------------------------------------------------------ vectors
struct int3;
struct uint3;
struct bool3 {
    bool x, y, z;
};
inline bool3 operator||(bool3 a, bool3 b) { return {a.x || b.x, a.y || b.y, a.z || b.z}; }
inline bool any(bool3 a) { return a.x || a.y || a.z; }

struct float3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    float3() = default;
    explicit float3(float s) : x(s), y(s), z(s) {}
    template <class A, class B, class C>
    float3(A a, B b, C c) : x((float)a), y((float)b), z((float)c) {}
    explicit float3(const uint3& v);
    explicit float3(const int3& v);
    float3& operator+=(const float3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    float3& operator-=(const float3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    float3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    float3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};
static_assert(sizeof(float3) == 12, "scalar layout");

inline float3 operator+(float3 a, float3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float3 operator-(float3 a, float3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float3 operator*(float3 a, float3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline float3 operator/(float3 a, float3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline float3 operator+(float3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
inline float3 operator-(float3 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
inline float3 operator*(float3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float3 operator/(float3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float3 operator+(float s, float3 a) { return {s + a.x, s + a.y, s + a.z}; }
inline float3 operator-(float s, float3 a) { return {s - a.x, s - a.y, s - a.z}; }
inline float3 operator*(float s, float3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline float3 operator-(float3 a) { return {-a.x, -a.y, -a.z}; }
inline bool3 operator<(float3 a, float3 b) { return {a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bool3 operator>(float3 a, float3 b) { return {a.x > b.x, a.y > b.y, a.z > b.z}; }

struct float4 {
    float x = 0.0f, y = 0.0f, z = 0.0f, w = 0.0f;
    float4() = default;
    template <class W>
    float4(float3 v, W w_) : x(v.x), y(v.y), z(v.z), w((float)w_) {}
    template <class A, class B, class C, class D>
    float4(A a, B b, C c, D d) : x((float)a), y((float)b), z((float)c), w((float)d) {}
    float3 xyz() const { return {x, y, z}; }
};

// Row-major: m[i] is row i and mul(M, v)[i] = dot(row i, v).
struct float4x4 {
    float m[4][4];
};
inline float4 mul(const float4x4& M, float4 v) {
    float r[4];
    for (int i = 0; i < 4; i++) r[i] = M.m[i][0] * v.x + M.m[i][1] * v.y + M.m[i][2] * v.z + M.m[i][3] * v.w;
    return {r[0], r[1], r[2], r[3]};
}

struct int3 {
    int x = 0, y = 0, z = 0;
    int3() = default;
    int3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit int3(const float3& v);
};
struct uint3 {
    uint x = 0, y = 0, z = 0;
    uint3() = default;
    template <class A, class B, class C>
    uint3(A a, B b, C c) : x((uint)a), y((uint)b), z((uint)c) {}
    explicit uint3(const float3& v);
};

// float -> int conversions that C++ leaves undefined abort.
inline int f2i(float f) {
    if (!(f >= -2147483648.0f && f < 2147483648.0f)) slang_shim::fault("float -> int out of range", (long long)f);
    return (int)f;
}
inline uint f2u(float f) {
    if (!(f >= 0.0f && f < 4294967296.0f)) slang_shim::fault("float -> uint out of range", (long long)f);
    return (uint)f;
}
inline float3::float3(const uint3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
inline float3::float3(const int3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
inline int3::int3(const float3& v) : x(f2i(v.x)), y(f2i(v.y)), z(f2i(v.z)) {}
inline uint3::uint3(const float3& v) : x(f2u(v.x)), y(f2u(v.y)), z(f2u(v.z)) {}

// Integer vector arithmetic wraps modulo 2^32 (two's complement), as on the GPU.
inline int3 operator+(int3 a, int3 b) {
    return {(int)((uint)a.x + (uint)b.x), (int)((uint)a.y + (uint)b.y), (int)((uint)a.z + (uint)b.z)};
}
inline uint3 operator+(int3 a, uint s) { return {(uint)a.x + s, (uint)a.y + s, (uint)a.z + s}; }
inline uint3 operator+(uint3 a, uint3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline uint3 operator%(uint3 a, uint s) { return {a.x % s, a.y % s, a.z % s}; }
inline uint3 operator/(uint3 a, uint s) { return {a.x / s, a.y / s, a.z / s}; }

// ------------------------------------------------------------------ intrinsics (float)
inline float floor(float a) { return __builtin_floorf(a); }
inline float3 floor(float3 a) { return {floor(a.x), floor(a.y), floor(a.z)}; }
inline float sqrt(float a) { return __builtin_sqrtf(a); }
inline float pow(float a, float b) { return __builtin_powf(a, b); }
inline float abs(float a) { return __builtin_fabsf(a); }
inline float min(float a, float b) { return a < b ? a : b; }
inline float max(float a, float b) { return a > b ? a : b; }
inline float3 min(float3 a, float3 b) { return {min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)}; }
inline float3 max(float3 a, float3 b) { return {max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)}; }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(float3 a) { return sqrt(dot(a, a)); }

// ------------------------------------------------------------------ atomics
inline void InterlockedAdd(uint& dst, uint v) { dst += v; }
inline void InterlockedAdd(uint& dst, uint v, uint& original) {
    original = dst;
    dst += v;
}

// ------------------------------------------------------------------ group barriers
// A group's threads run as fibers; GroupMemoryBarrierWithGroupSync returns control to the
// scheduler, which resumes every thread up to its next barrier before any passes it. A fiber is
// entered once through its ucontext and afterwards switched with _setjmp/_longjmp (no signal-mask
// system call per switch). Each host thread has its own scheduler, so different workgroups can
// run on different host threads.
namespace slang_shim {
struct FiberGroup {
    static constexpr int kMaxThreads = 1024;
    static constexpr size_t kStack = 64 * 1024;
    jmp_buf main_jb;
    jmp_buf jb[kMaxThreads];
    ucontext_t ctx[kMaxThreads];
    bool done[kMaxThreads];
    bool started[kMaxThreads];
    char* stacks = nullptr;
    int current = -1;
    void (*body)(int thread) = nullptr;
    ~FiberGroup() { std::free(stacks); }
};
inline FiberGroup& fibers() {
    static thread_local FiberGroup g;
    return g;
}
inline void fiber_entry() {
    FiberGroup& g = fibers();
    const int t = g.current;
    g.body(t);
    g.done[t] = true;
    _longjmp(g.main_jb, 1);
}
// Runs body(t) for t in [0, threads) as one workgroup with barrier semantics.
inline void run_group(int threads, void (*body)(int)) {
    FiberGroup& g = fibers();
    if (threads > FiberGroup::kMaxThreads) fault("workgroup too large", threads);
    if (!g.stacks) g.stacks = static_cast<char*>(std::malloc(FiberGroup::kStack * FiberGroup::kMaxThreads));
    g.body = body;
    for (int t = 0; t < threads; t++) {
        g.done[t] = false;
        g.started[t] = false;
    }
    for (;;) {
        int live = 0;
        for (int t = 0; t < threads; t++) {
            if (g.done[t]) continue;
            live++;
            g.current = t;
            if (!_setjmp(g.main_jb)) {
                if (!g.started[t]) {
                    g.started[t] = true;
                    getcontext(&g.ctx[t]);
                    g.ctx[t].uc_stack.ss_sp = g.stacks + FiberGroup::kStack * (size_t)t;
                    g.ctx[t].uc_stack.ss_size = FiberGroup::kStack;
                    g.ctx[t].uc_link = nullptr;
                    makecontext(&g.ctx[t], fiber_entry, 0);
                    setcontext(&g.ctx[t]);
                } else {
                    _longjmp(g.jb[t], 1);
                }
            }
        }
        if (!live) break;
    }
    g.current = -1;
}
}  // namespace slang_shim

inline void GroupMemoryBarrierWithGroupSync() {
    slang_shim::FiberGroup& g = slang_shim::fibers();
    if (g.current < 0) slang_shim::fault("group barrier outside a workgroup");
    if (!_setjmp(g.jb[g.current])) _longjmp(g.main_jb, 1);
}
