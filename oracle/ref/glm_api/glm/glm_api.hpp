// glm_api.hpp — the subset of the glm 1.0.1 API that AdaptiveSph's cuda/ library uses, restated for compiling that
// library as a checker (TEST INFRASTRUCTURE ONLY: it builds oracle/_ref, never the product). glm itself is a
// third-party dependency fetched by the reference's CMake (Dependencies.cmake:9) and absent here.
//
// What is restated, from glm's documented semantics: vec3 / vec4 of float and ivec3 / uvec3 of int, with
// componentwise arithmetic against vectors and scalars, converting constructors (truncation to int, dropping or
// appending w), indexing; dot (vec4: (x*y + ... ) summed as (p.x + p.y) + (p.z + p.w); vec3: p.x + p.y + p.z, the
// order of glm's generic implementation), length = sqrt(dot(v, v)), sqrt, min / max ((b < a) ? b : a and
// (a < b) ? b : a), clamp = min(max(x, lo), hi), ceil, compMin. Layout: tightly packed floats, 4-byte aligned (glm's
// default, no SIMD alignment), so the reference's kernels load them as it does with glm.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define GLM_API_FN __host__ __device__ inline
#else
#define GLM_API_FN inline
#endif

namespace glm {

template <class T>
struct tvec3;
template <class T>
struct tvec4;

template <class T>
struct tvec3 {
    T x = T(0), y = T(0), z = T(0);
    tvec3() = default;
    GLM_API_FN explicit tvec3(T s) : x(s), y(s), z(s) {}
    GLM_API_FN tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    template <class U>
    GLM_API_FN explicit tvec3(const tvec3<U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
    template <class U>
    GLM_API_FN explicit tvec3(const tvec4<U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
    GLM_API_FN T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    GLM_API_FN const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    GLM_API_FN tvec3& operator+=(const tvec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    GLM_API_FN tvec3& operator-=(const tvec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    GLM_API_FN tvec3& operator*=(const tvec3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    GLM_API_FN tvec3& operator/=(const tvec3& o) { x /= o.x; y /= o.y; z /= o.z; return *this; }
    GLM_API_FN tvec3& operator+=(T s) { x += s; y += s; z += s; return *this; }
    GLM_API_FN tvec3& operator-=(T s) { x -= s; y -= s; z -= s; return *this; }
    GLM_API_FN tvec3& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
    GLM_API_FN tvec3& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }
};

template <class T>
struct tvec4 {
    T x = T(0), y = T(0), z = T(0), w = T(0);
    tvec4() = default;
    GLM_API_FN explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
    GLM_API_FN tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    GLM_API_FN tvec4(const tvec3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    GLM_API_FN T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    GLM_API_FN const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    GLM_API_FN tvec4& operator+=(const tvec4& o) { x += o.x; y += o.y; z += o.z; w += o.w; return *this; }
    GLM_API_FN tvec4& operator-=(const tvec4& o) { x -= o.x; y -= o.y; z -= o.z; w -= o.w; return *this; }
    GLM_API_FN tvec4& operator*=(const tvec4& o) { x *= o.x; y *= o.y; z *= o.z; w *= o.w; return *this; }
    GLM_API_FN tvec4& operator/=(const tvec4& o) { x /= o.x; y /= o.y; z /= o.z; w /= o.w; return *this; }
    GLM_API_FN tvec4& operator+=(T s) { x += s; y += s; z += s; w += s; return *this; }
    GLM_API_FN tvec4& operator-=(T s) { x -= s; y -= s; z -= s; w -= s; return *this; }
    GLM_API_FN tvec4& operator*=(T s) { x *= s; y *= s; z *= s; w *= s; return *this; }
    GLM_API_FN tvec4& operator/=(T s) { x /= s; y /= s; z /= s; w /= s; return *this; }
};

// componentwise binary operators: vector-vector, vector-scalar, scalar-vector
#define GLM_API_BINOP(OP)                                                                                        \
    template <class T>                                                                                           \
    GLM_API_FN tvec3<T> operator OP(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z); } \
    template <class T>                                                                                           \
    GLM_API_FN tvec3<T> operator OP(const tvec3<T>& a, T s) { return tvec3<T>(a.x OP s, a.y OP s, a.z OP s); }   \
    template <class T>                                                                                           \
    GLM_API_FN tvec3<T> operator OP(T s, const tvec3<T>& a) { return tvec3<T>(s OP a.x, s OP a.y, s OP a.z); }   \
    template <class T>                                                                                           \
    GLM_API_FN tvec4<T> operator OP(const tvec4<T>& a, const tvec4<T>& b) {                                      \
        return tvec4<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w);                                         \
    }                                                                                                            \
    template <class T>                                                                                           \
    GLM_API_FN tvec4<T> operator OP(const tvec4<T>& a, T s) { return tvec4<T>(a.x OP s, a.y OP s, a.z OP s, a.w OP s); } \
    template <class T>                                                                                           \
    GLM_API_FN tvec4<T> operator OP(T s, const tvec4<T>& a) { return tvec4<T>(s OP a.x, s OP a.y, s OP a.z, s OP a.w); }
GLM_API_BINOP(+)
GLM_API_BINOP(-)
GLM_API_BINOP(*)
GLM_API_BINOP(/)
#undef GLM_API_BINOP

template <class T>
GLM_API_FN tvec3<T> operator-(const tvec3<T>& a) { return tvec3<T>(-a.x, -a.y, -a.z); }
template <class T>
GLM_API_FN tvec4<T> operator-(const tvec4<T>& a) { return tvec4<T>(-a.x, -a.y, -a.z, -a.w); }
template <class T>
GLM_API_FN bool operator==(const tvec3<T>& a, const tvec3<T>& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <class T>
GLM_API_FN bool operator==(const tvec4<T>& a, const tvec4<T>& b) {
    return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
}

using vec3 = tvec3<float>;
using vec4 = tvec4<float>;
using ivec3 = tvec3<int>;
using uvec3 = tvec3<unsigned int>;

GLM_API_FN float dot(const vec4& a, const vec4& b) {
    const vec4 p = a * b;
    return (p.x + p.y) + (p.z + p.w);
}
GLM_API_FN float dot(const vec3& a, const vec3& b) {
    const vec3 p = a * b;
    return p.x + p.y + p.z;
}
GLM_API_FN float sqrt(float x) { return ::sqrtf(x); }
GLM_API_FN float length(const vec4& v) { return glm::sqrt(glm::dot(v, v)); }
GLM_API_FN float length(const vec3& v) { return glm::sqrt(glm::dot(v, v)); }

template <class T>
GLM_API_FN T min(T a, T b) { return (b < a) ? b : a; }
template <class T>
GLM_API_FN T max(T a, T b) { return (a < b) ? b : a; }
template <class T>
GLM_API_FN tvec3<T> min(const tvec3<T>& a, const tvec3<T>& b) {
    return tvec3<T>(glm::min(a.x, b.x), glm::min(a.y, b.y), glm::min(a.z, b.z));
}
template <class T>
GLM_API_FN tvec3<T> max(const tvec3<T>& a, const tvec3<T>& b) {
    return tvec3<T>(glm::max(a.x, b.x), glm::max(a.y, b.y), glm::max(a.z, b.z));
}
template <class T>
GLM_API_FN tvec3<T> min(const tvec3<T>& a, T b) { return glm::min(a, tvec3<T>(b)); }
template <class T>
GLM_API_FN tvec3<T> max(const tvec3<T>& a, T b) { return glm::max(a, tvec3<T>(b)); }
template <class T>
GLM_API_FN tvec3<T> clamp(const tvec3<T>& x, const tvec3<T>& lo, const tvec3<T>& hi) {
    return glm::min(glm::max(x, lo), hi);
}
template <class T>
GLM_API_FN T clamp(T x, T lo, T hi) { return glm::min(glm::max(x, lo), hi); }
GLM_API_FN vec3 ceil(const vec3& v) { return vec3(::ceilf(v.x), ::ceilf(v.y), ::ceilf(v.z)); }
template <class T>
GLM_API_FN T compMin(const tvec3<T>& v) { return glm::min(glm::min(v.x, v.y), v.z); }

}  // namespace glm
