// TEST INFRASTRUCTURE ONLY: the few GLM types and functions that cuda_voxelizer's voxelize.cu and
// util.h use, so that the reference voxelizer kernel compiles from its own sources without the
// GLM package (glm 0.9.9.8, which the reference downloads at configure time and does not vendor).
//
// Each function follows GLM's published definition and operation order, since the compiler's
// contraction of multiplies and adds into FMAs depends on the expression's structure:
//   dot(a, b)       tmp = a * b; tmp.x + tmp.y (+ tmp.z)   (left to right)
//   cross(x, y)     (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y)
//   normalize(x)    x * inversesqrt(dot(x, x)),  inversesqrt(s) = 1 / sqrt(s)
//   min(x, y)       (y < x) ? y : x       max(x, y)   (x < y) ? y : x     (per component)
//   clamp(x, a, b)  min(max(x, a), b)
//   vec<int> from vec<float>: static_cast per component (truncation)
#pragma once

#include <cmath>
#include <cstddef>

#ifdef __CUDACC__
#define GLMS_FN __host__ __device__ inline
#else
#define GLMS_FN inline
#endif

namespace glm {

template <typename T>
struct tvec2 {
    T x, y;
    GLMS_FN tvec2() : x(0), y(0) {}
    template <typename A, typename B>
    GLMS_FN tvec2(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
    GLMS_FN T& operator[](int i) { return i == 0 ? x : y; }
    GLMS_FN const T& operator[](int i) const { return i == 0 ? x : y; }
};

template <typename T>
struct tvec3 {
    T x, y, z;
    GLMS_FN tvec3() : x(0), y(0), z(0) {}
    GLMS_FN explicit tvec3(T s) : x(s), y(s), z(s) {}
    template <typename A, typename B, typename C>
    GLMS_FN tvec3(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
    template <typename U>
    GLMS_FN tvec3(const tvec3<U>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
    template <typename U>
    GLMS_FN tvec3& operator=(const tvec3<U>& v) {
        x = static_cast<T>(v.x);
        y = static_cast<T>(v.y);
        z = static_cast<T>(v.z);
        return *this;
    }
    GLMS_FN T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    GLMS_FN const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    GLMS_FN tvec3& operator+=(const tvec3& v) {
        x += v.x;
        y += v.y;
        z += v.z;
        return *this;
    }
    GLMS_FN tvec3& operator-=(const tvec3& v) {
        x -= v.x;
        y -= v.y;
        z -= v.z;
        return *this;
    }
};

using vec2 = tvec2<float>;
using vec3 = tvec3<float>;
using ivec3 = tvec3<int>;
using uvec3 = tvec3<unsigned int>;

template <typename T> GLMS_FN tvec2<T> operator*(const tvec2<T>& a, const tvec2<T>& b) { return tvec2<T>(a.x * b.x, a.y * b.y); }
template <typename T> GLMS_FN tvec2<T> operator-(const tvec2<T>& v) { return tvec2<T>(-v.x, -v.y); }

template <typename T> GLMS_FN tvec3<T> operator+(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> GLMS_FN tvec3<T> operator-(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> GLMS_FN tvec3<T> operator*(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename T> GLMS_FN tvec3<T> operator/(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <typename T> GLMS_FN tvec3<T> operator*(const tvec3<T>& a, T s) { return tvec3<T>(a.x * s, a.y * s, a.z * s); }
template <typename T> GLMS_FN tvec3<T> operator-(const tvec3<T>& v) { return tvec3<T>(-v.x, -v.y, -v.z); }

template <typename T> GLMS_FN T min(T x, T y) { return (y < x) ? y : x; }
template <typename T> GLMS_FN T max(T x, T y) { return (x < y) ? y : x; }
template <typename T> GLMS_FN tvec3<T> min(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
template <typename T> GLMS_FN tvec3<T> max(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
template <typename T> GLMS_FN tvec3<T> clamp(const tvec3<T>& x, const tvec3<T>& lo, const tvec3<T>& hi) { return min(max(x, lo), hi); }

template <typename T> GLMS_FN T dot(const tvec2<T>& a, const tvec2<T>& b) {
    const tvec2<T> t = a * b;
    return t.x + t.y;
}
template <typename T> GLMS_FN T dot(const tvec3<T>& a, const tvec3<T>& b) {
    const tvec3<T> t = a * b;
    return t.x + t.y + t.z;
}
template <typename T> GLMS_FN tvec3<T> cross(const tvec3<T>& x, const tvec3<T>& y) {
    return tvec3<T>(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}
GLMS_FN float inversesqrt(float s) { return 1.0f / sqrtf(s); }
template <typename T> GLMS_FN tvec3<T> normalize(const tvec3<T>& x) { return x * inversesqrt(dot(x, x)); }

}  // namespace glm
