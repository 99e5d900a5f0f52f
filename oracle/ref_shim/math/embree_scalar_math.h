// embree_scalar_math.h -- scalar stand-in for the part of Embree's vector math
// (namespace embree: Vec2, Vec3, Vec4, Vec3fa and the scalar helpers) that
// Lantern's sources use through math/vector_types.h.
//
// TEST INFRASTRUCTURE ONLY: used to compile the reference integrator as the CPU
// oracle and CPU baseline (oracle/build_ref.sh). Embree's own headers are SSE
// (third_party/embree/common/math/vec3fa.h) and do not compile on aarch64, so
// this file gives the same interface in portable scalar C++.
//
// Arithmetic is plain IEEE single precision with no fused multiply-add; dot
// products are (x*x + y*y) + z*z; normalize(a) = a * (1 / sqrt(dot(a, a)));
// Embree's approximate rcp/rsqrt become exact divisions. The C restatement in
// oracle/lt_oracle.c uses the same definitions, which is what lets the two
// agree bit for bit.
#pragma once

#include <cmath>
#include <cstddef>
#include <iostream>
#include <limits>

namespace embree {

struct ZeroTy { __inline operator float() const { return 0.0f; } };
struct OneTy { __inline operator float() const { return 1.0f; } };
struct PosInfTy { __inline operator float() const { return std::numeric_limits<float>::infinity(); } };
struct NegInfTy { __inline operator float() const { return -std::numeric_limits<float>::infinity(); } };
static const ZeroTy zero = ZeroTy();
static const OneTy one = OneTy();
static const PosInfTy inf = PosInfTy();
static const PosInfTy pos_inf = PosInfTy();
static const NegInfTy neg_inf = NegInfTy();

inline float rcp(float x) { return 1.0f / x; }
inline float rsqrt(float x) { return 1.0f / std::sqrt(x); }
inline float sqr(float x) { return x * x; }
inline float madd(float a, float b, float c) { return a * b + c; }
inline float msub(float a, float b, float c) { return a * b - c; }
inline float abs(float x) { return std::fabs(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float exp(float x) { return std::exp(x); }
inline float log(float x) { return std::log(x); }
inline float min(float a, float b) { return a < b ? a : b; }
inline float max(float a, float b) { return a > b ? a : b; }

// ---------------------------------------------------------------- Vec2
template <typename T> struct Vec2 {
    T x, y;
    Vec2() : x(T()), y(T()) {}
    explicit Vec2(const T &a) : x(a), y(a) {}
    Vec2(const T &x_, const T &y_) : x(x_), y(y_) {}
    Vec2(ZeroTy) : x(T(0)), y(T(0)) {}
    const T &operator[](size_t i) const { return (&x)[i]; }
    T &operator[](size_t i) { return (&x)[i]; }
};
template <typename T> Vec2<T> operator+(const Vec2<T> &a, const Vec2<T> &b) { return Vec2<T>(a.x + b.x, a.y + b.y); }
template <typename T> Vec2<T> operator-(const Vec2<T> &a, const Vec2<T> &b) { return Vec2<T>(a.x - b.x, a.y - b.y); }
template <typename T> Vec2<T> operator*(const Vec2<T> &a, const T &b) { return Vec2<T>(a.x * b, a.y * b); }
template <typename T> Vec2<T> operator*(const T &a, const Vec2<T> &b) { return Vec2<T>(a * b.x, a * b.y); }
template <typename T> Vec2<T> operator*(const Vec2<T> &a, const Vec2<T> &b) { return Vec2<T>(a.x * b.x, a.y * b.y); }
template <typename T> Vec2<T> operator/(const Vec2<T> &a, const T &b) { return Vec2<T>(a.x / b, a.y / b); }

// ---------------------------------------------------------------- Vec3
struct Vec3fa;

template <typename T> struct Vec3 {
    T x, y, z;
    Vec3() : x(T()), y(T()), z(T()) {}
    explicit Vec3(const T &a) : x(a), y(a), z(a) {}
    Vec3(const T &x_, const T &y_, const T &z_) : x(x_), y(y_), z(z_) {}
    Vec3(ZeroTy) : x(T(0)), y(T(0)), z(T(0)) {}
    Vec3(OneTy) : x(T(1)), y(T(1)), z(T(1)) {}
    inline Vec3(const Vec3fa &a);
    const T &operator[](size_t i) const { return (&x)[i]; }
    T &operator[](size_t i) { return (&x)[i]; }
};

template <typename T> Vec3<T> operator-(const Vec3<T> &a) { return Vec3<T>(-a.x, -a.y, -a.z); }
template <typename T> Vec3<T> operator+(const Vec3<T> &a, const Vec3<T> &b) { return Vec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> Vec3<T> operator-(const Vec3<T> &a, const Vec3<T> &b) { return Vec3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> Vec3<T> operator*(const Vec3<T> &a, const Vec3<T> &b) { return Vec3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename T> Vec3<T> operator*(const Vec3<T> &a, const T &b) { return Vec3<T>(a.x * b, a.y * b, a.z * b); }
template <typename T> Vec3<T> operator*(const T &a, const Vec3<T> &b) { return Vec3<T>(a * b.x, a * b.y, a * b.z); }
template <typename T> Vec3<T> operator/(const Vec3<T> &a, const Vec3<T> &b) { return Vec3<T>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <typename T> Vec3<T> operator/(const Vec3<T> &a, const T &b) { return Vec3<T>(a.x / b, a.y / b, a.z / b); }
template <typename T> Vec3<T> &operator+=(Vec3<T> &a, const Vec3<T> &b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
template <typename T> Vec3<T> &operator-=(Vec3<T> &a, const Vec3<T> &b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
template <typename T> Vec3<T> &operator*=(Vec3<T> &a, const T &b) { a.x *= b; a.y *= b; a.z *= b; return a; }
template <typename T> Vec3<T> &operator/=(Vec3<T> &a, const T &b) { a.x /= b; a.y /= b; a.z /= b; return a; }
template <typename T> bool operator==(const Vec3<T> &a, const Vec3<T> &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <typename T> T dot(const Vec3<T> &a, const Vec3<T> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> T length(const Vec3<T> &a) { return std::sqrt(dot(a, a)); }
template <typename T> T sqr_length(const Vec3<T> &a) { return dot(a, a); }
template <typename T> Vec3<T> normalize(const Vec3<T> &a) { return a * (T(1) / std::sqrt(dot(a, a))); }
template <typename T> Vec3<T> cross(const Vec3<T> &a, const Vec3<T> &b) {
    return Vec3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename T> Vec3<T> exp(const Vec3<T> &a) { return Vec3<T>(std::exp(a.x), std::exp(a.y), std::exp(a.z)); }
template <typename T> Vec3<T> log(const Vec3<T> &a) { return Vec3<T>(std::log(a.x), std::log(a.y), std::log(a.z)); }
template <typename T> std::ostream &operator<<(std::ostream &o, const Vec3<T> &a) {
    return o << "(" << a.x << ", " << a.y << ", " << a.z << ")";
}

// ---------------------------------------------------------------- Vec3fa
// 16-byte vector with a fourth lane; Vec3fa(x, y, z) copies z into the fourth
// lane as Embree's _mm_set_ps(z, z, y, x) does.
struct alignas(16) Vec3fa {
    float x, y, z, w;
    Vec3fa() : x(0), y(0), z(0), w(0) {}
    explicit Vec3fa(float a) : x(a), y(a), z(a), w(a) {}
    Vec3fa(float x_, float y_, float z_) : x(x_), y(y_), z(z_), w(z_) {}
    Vec3fa(float x_, float y_, float z_, float w_) : x(x_), y(y_), z(z_), w(w_) {}
    Vec3fa(const Vec3<float> &o) : x(o.x), y(o.y), z(o.z), w(o.z) {}
    Vec3fa(const Vec3fa &o, float w_) : x(o.x), y(o.y), z(o.z), w(w_) {}
    Vec3fa(ZeroTy) : x(0), y(0), z(0), w(0) {}
    Vec3fa(OneTy) : x(1), y(1), z(1), w(1) {}
    Vec3fa(PosInfTy) : x(pos_inf), y(pos_inf), z(pos_inf), w(pos_inf) {}
    const float &operator[](size_t i) const { return (&x)[i]; }
    float &operator[](size_t i) { return (&x)[i]; }
};

template <typename T> inline Vec3<T>::Vec3(const Vec3fa &a) : x(a.x), y(a.y), z(a.z) {}

inline Vec3fa operator-(const Vec3fa &a) { return Vec3fa(-a.x, -a.y, -a.z, -a.w); }
inline Vec3fa operator+(const Vec3fa &a, const Vec3fa &b) { return Vec3fa(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline Vec3fa operator-(const Vec3fa &a, const Vec3fa &b) { return Vec3fa(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline Vec3fa operator*(const Vec3fa &a, const Vec3fa &b) { return Vec3fa(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline Vec3fa operator*(const Vec3fa &a, float b) { return Vec3fa(a.x * b, a.y * b, a.z * b, a.w * b); }
inline Vec3fa operator*(float a, const Vec3fa &b) { return Vec3fa(a * b.x, a * b.y, a * b.z, a * b.w); }
inline Vec3fa operator/(const Vec3fa &a, const Vec3fa &b) { return Vec3fa(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }
inline Vec3fa operator/(const Vec3fa &a, float b) { return Vec3fa(a.x / b, a.y / b, a.z / b, a.w / b); }
inline Vec3fa &operator+=(Vec3fa &a, const Vec3fa &b) { return a = a + b; }
inline Vec3fa &operator-=(Vec3fa &a, const Vec3fa &b) { return a = a - b; }
inline Vec3fa &operator*=(Vec3fa &a, float b) { return a = a * b; }
inline Vec3fa &operator/=(Vec3fa &a, float b) { return a = a / b; }
inline bool operator==(const Vec3fa &a, const Vec3fa &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline float dot(const Vec3fa &a, const Vec3fa &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3fa cross(const Vec3fa &a, const Vec3fa &b) {
    return Vec3fa(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float sqr_length(const Vec3fa &a) { return dot(a, a); }
inline float length(const Vec3fa &a) { return std::sqrt(dot(a, a)); }
inline float rcp_length(const Vec3fa &a) { return 1.0f / std::sqrt(dot(a, a)); }
inline Vec3fa normalize(const Vec3fa &a) { return a * (1.0f / std::sqrt(dot(a, a))); }
inline float distance(const Vec3fa &a, const Vec3fa &b) { return length(a - b); }
inline Vec3fa abs(const Vec3fa &a) { return Vec3fa(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z), std::fabs(a.w)); }
inline Vec3fa exp(const Vec3fa &a) { return Vec3fa(std::exp(a.x), std::exp(a.y), std::exp(a.z), std::exp(a.w)); }
inline Vec3fa log(const Vec3fa &a) { return Vec3fa(std::log(a.x), std::log(a.y), std::log(a.z), std::log(a.w)); }
inline Vec3fa min(const Vec3fa &a, const Vec3fa &b) { return Vec3fa(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z), min(a.w, b.w)); }
inline Vec3fa max(const Vec3fa &a, const Vec3fa &b) { return Vec3fa(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
inline std::ostream &operator<<(std::ostream &o, const Vec3fa &a) {
    return o << "(" << a.x << ", " << a.y << ", " << a.z << ")";
}

// ---------------------------------------------------------------- Vec4
template <typename T> struct Vec4 {
    T x, y, z, w;
    Vec4() : x(T()), y(T()), z(T()), w(T()) {}
    explicit Vec4(const T &a) : x(a), y(a), z(a), w(a) {}
    Vec4(const T &x_, const T &y_, const T &z_, const T &w_) : x(x_), y(y_), z(z_), w(w_) {}
    Vec4(const Vec3<T> &xyz_, const T &w_) : x(xyz_.x), y(xyz_.y), z(xyz_.z), w(w_) {}
    Vec4(const Vec3fa &a, const T &w_) : x(a.x), y(a.y), z(a.z), w(w_) {}
    Vec4(const Vec3fa &a) : x(a.x), y(a.y), z(a.z), w(a.w) {}
    Vec4(ZeroTy) : x(T(0)), y(T(0)), z(T(0)), w(T(0)) {}
    Vec4(OneTy) : x(T(1)), y(T(1)), z(T(1)), w(T(1)) {}
    operator Vec3fa() const { return Vec3fa(x, y, z, w); }
    Vec3<T> xyz() const { return Vec3<T>(x, y, z); }
    const T &operator[](size_t i) const { return (&x)[i]; }
    T &operator[](size_t i) { return (&x)[i]; }
};
typedef Vec4<float> Vec4f;
template <typename T> Vec4<T> operator-(const Vec4<T> &a) { return Vec4<T>(-a.x, -a.y, -a.z, -a.w); }
template <typename T> Vec4<T> operator+(const Vec4<T> &a) { return a; }
template <typename T> Vec4<T> operator+(const Vec4<T> &a, const Vec4<T> &b) { return Vec4<T>(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
template <typename T> Vec4<T> operator-(const Vec4<T> &a, const Vec4<T> &b) { return Vec4<T>(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
template <typename T> Vec4<T> operator*(const Vec4<T> &a, const Vec4<T> &b) { return Vec4<T>(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
template <typename T> Vec4<T> operator*(const T &a, const Vec4<T> &b) { return Vec4<T>(a * b.x, a * b.y, a * b.z, a * b.w); }
template <typename T> Vec4<T> operator*(const Vec4<T> &a, const T &b) { return Vec4<T>(a.x * b, a.y * b, a.z * b, a.w * b); }
template <typename T> Vec4<T> operator/(const Vec4<T> &a, const T &b) { return Vec4<T>(a.x / b, a.y / b, a.z / b, a.w / b); }
template <typename T> bool operator==(const Vec4<T> &a, const Vec4<T> &b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }
template <typename T> bool operator!=(const Vec4<T> &a, const Vec4<T> &b) { return !(a == b); }
template <typename T> T dot(const Vec4<T> &a, const Vec4<T> &b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <typename T> Vec4<T> normalize(const Vec4<T> &a) { return a * (T(1) / std::sqrt(dot(a, a))); }
template <typename T> std::ostream &operator<<(std::ostream &o, const Vec4<T> &a) {
    return o << "(" << a.x << ", " << a.y << ", " << a.z << ", " << a.w << ")";
}

}  // namespace embree

#ifndef __forceinline
#define __forceinline inline __attribute__((always_inline))
#endif
