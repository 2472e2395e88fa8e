// Project-written stand-in for the small part of glm 1.0.1 that the reference's CPU volume-map
// code uses (src/util/: geometry, mesh_bvh, mesh_pseudonormals, mesh_sdf, discretization,
// gaussian_quadrature, kernel, volume_map), so that code compiles here as a checker for the
// oracle (test infrastructure; glm itself is not in this image).
//
// Semantics follow glm's: vec2/vec3 templates over the component type with implicit conversions
// between component types, component-wise operators between a vector and a vector or a scalar of
// the same component type, dot = (x*x' + y*y') + z*z', length = sqrt(dot), normalize = v *
// (1 / sqrt(dot(v, v))) (glm's inversesqrt), cross in glm's operand order, compMul = (x*y)*z.
#pragma once

#include <cmath>
#include <cstdint>

namespace glm {

template <class T>
struct tvec2 {
    T x, y;
    constexpr tvec2() : x(0), y(0) {}
    explicit constexpr tvec2(T s) : x(s), y(s) {}
    template <class A, class B>
    constexpr tvec2(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
};

template <class T>
struct tvec3 {
    T x, y, z;
    constexpr tvec3() : x(0), y(0), z(0) {}
    explicit constexpr tvec3(T s) : x(s), y(s), z(s) {}
    template <class A, class B, class C>
    constexpr tvec3(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
    template <class U>
    constexpr tvec3(const tvec3<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    tvec3& operator+=(const tvec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    tvec3& operator-=(const tvec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    tvec3& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
    tvec3& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }
};

template <class T> tvec3<T> operator+(const tvec3<T>& a, const tvec3<T>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> tvec3<T> operator-(const tvec3<T>& a, const tvec3<T>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> tvec3<T> operator*(const tvec3<T>& a, const tvec3<T>& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> tvec3<T> operator/(const tvec3<T>& a, const tvec3<T>& b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> tvec3<T> operator+(const tvec3<T>& a, T s) { return {a.x + s, a.y + s, a.z + s}; }
template <class T> tvec3<T> operator-(const tvec3<T>& a, T s) { return {a.x - s, a.y - s, a.z - s}; }
template <class T> tvec3<T> operator*(const tvec3<T>& a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> tvec3<T> operator/(const tvec3<T>& a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> tvec3<T> operator+(T s, const tvec3<T>& a) { return {s + a.x, s + a.y, s + a.z}; }
template <class T> tvec3<T> operator-(T s, const tvec3<T>& a) { return {s - a.x, s - a.y, s - a.z}; }
template <class T> tvec3<T> operator*(T s, const tvec3<T>& a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> tvec3<T> operator-(const tvec3<T>& a) { return {-a.x, -a.y, -a.z}; }
template <class T> bool operator==(const tvec3<T>& a, const tvec3<T>& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <class T> bool operator!=(const tvec3<T>& a, const tvec3<T>& b) { return !(a == b); }

using vec2 = tvec2<float>;
using vec3 = tvec3<float>;
using dvec3 = tvec3<double>;
using uvec3 = tvec3<uint32_t>;
using ivec3 = tvec3<int32_t>;
using bvec3 = tvec3<bool>;

template <class T> T dot(const tvec3<T>& a, const tvec3<T>& b) {
    const tvec3<T> t = a * b;
    return (t.x + t.y) + t.z;
}
template <class T> tvec3<T> cross(const tvec3<T>& x, const tvec3<T>& y) {
    return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
}
template <class T> T length(const tvec3<T>& v) { return std::sqrt(dot(v, v)); }
template <class T> T length2(const tvec3<T>& v) { return dot(v, v); }
template <class T> tvec3<T> normalize(const tvec3<T>& v) { return v * (static_cast<T>(1) / std::sqrt(dot(v, v))); }
template <class T> tvec3<T> abs(const tvec3<T>& v) { return {std::abs(v.x), std::abs(v.y), std::abs(v.z)}; }
template <class T> T abs(T v) { return std::abs(v); }
template <class T> tvec3<T> floor(const tvec3<T>& v) { return {std::floor(v.x), std::floor(v.y), std::floor(v.z)}; }
template <class T> tvec3<T> min(const tvec3<T>& a, const tvec3<T>& b) {
    return {b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z};
}
template <class T> tvec3<T> max(const tvec3<T>& a, const tvec3<T>& b) {
    return {a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z};
}
template <class T> T compMul(const tvec3<T>& v) { return (v.x * v.y) * v.z; }
template <class T> bvec3 lessThanEqual(const tvec3<T>& a, const tvec3<T>& b) { return {a.x <= b.x, a.y <= b.y, a.z <= b.z}; }
template <class T> bvec3 greaterThanEqual(const tvec3<T>& a, const tvec3<T>& b) { return {a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bool all(const bvec3& v) { return v.x && v.y && v.z; }
template <class T> T* value_ptr(tvec3<T>& v) { return &v.x; }
template <class T> const T* value_ptr(const tvec3<T>& v) { return &v.x; }
template <class T> constexpr T zero() { return T(0); }
template <class T> constexpr T pi() { return T(3.14159265358979323846264338327950288); }

}  // namespace glm
