// glm-subset shim used ONLY to compile the reference software raster sources
// into the test oracle (oracle/_ref). It is written from glm's documented
// semantics (column-major mat4, component-wise vector arithmetic) and covers
// only the symbols those sources use. It is test infrastructure, never part of
// the shipped library.
//
// Summation orders follow the documented glm definitions:
//   mat4 * vec4  = (m[0]*v.x + m[1]*v.y) + (m[2]*v.z + m[3]*v.w)
//   mat4 * mat4  : column j = ((A0*b[j].x + A1*b[j].y) + A2*b[j].z) + A3*b[j].w
//   dot(a, b)    = a.x*b.x + a.y*b.y (+ ...), summed left to right
#ifndef ORACLE_GLM_SHIM_GLM_HPP
#define ORACLE_GLM_SHIM_GLM_HPP

#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <algorithm>

namespace glm {

template <typename T>
struct tvec2 {
  union { T x; T r; };
  union { T y; T g; };
  tvec2() : x(0), y(0) {}
  explicit tvec2(T s) : x(s), y(s) {}
  tvec2(T a, T b) : x(a), y(b) {}
  template <typename U>
  explicit tvec2(const tvec2<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)) {}
  T& operator[](int i) { return i == 0 ? x : y; }
  const T& operator[](int i) const { return i == 0 ? x : y; }
};

template <typename T>
struct tvec3 {
  union { T x; T r; };
  union { T y; T g; };
  union { T z; T b; };
  tvec3() : x(0), y(0), z(0) {}
  explicit tvec3(T s) : x(s), y(s), z(s) {}
  tvec3(T a, T b_, T c) : x(a), y(b_), z(c) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <typename T>
struct tvec4 {
  union { T x; T r; };
  union { T y; T g; };
  union { T z; T b; };
  union { T w; T a; };
  tvec4() : x(0), y(0), z(0), w(0) {}
  explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
  tvec4(T a_, T b_, T c, T d) : x(a_), y(b_), z(c), w(d) {}
  tvec4(const tvec3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  const T& operator[](int i) const {
    return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w));
  }
};

// ---- component-wise arithmetic -------------------------------------------
#define SHIM_VEC_OPS(V, N)                                                  \
  template <typename T>                                                     \
  inline V<T> operator+(const V<T>& a, const V<T>& b) {                     \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] + b[i]; return r;       \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T> operator-(const V<T>& a, const V<T>& b) {                     \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] - b[i]; return r;       \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T> operator*(const V<T>& a, const V<T>& b) {                     \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] * b[i]; return r;       \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T> operator/(const V<T>& a, const V<T>& b) {                     \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] / b[i]; return r;       \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T> operator*(const V<T>& a, T s) {                               \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] * s; return r;          \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T> operator*(T s, const V<T>& a) {                               \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = s * a[i]; return r;          \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T> operator/(const V<T>& a, T s) {                               \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] / s; return r;          \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T> operator+(const V<T>& a, T s) {                               \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] + s; return r;          \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T> operator-(const V<T>& a, T s) {                               \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] - s; return r;          \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T> operator-(const V<T>& a) {                                    \
    V<T> r; for (int i = 0; i < N; ++i) r[i] = -a[i]; return r;             \
  }                                                                         \
  template <typename T>                                                     \
  inline V<T>& operator+=(V<T>& a, const V<T>& b) { a = a + b; return a; }  \
  template <typename T>                                                     \
  inline V<T>& operator-=(V<T>& a, const V<T>& b) { a = a - b; return a; }  \
  template <typename T>                                                     \
  inline V<T>& operator*=(V<T>& a, const V<T>& b) { a = a * b; return a; }  \
  template <typename T>                                                     \
  inline V<T>& operator*=(V<T>& a, T s) { a = a * s; return a; }            \
  template <typename T>                                                     \
  inline V<T>& operator/=(V<T>& a, T s) { a = a / s; return a; }            \
  template <typename T>                                                     \
  inline bool operator==(const V<T>& a, const V<T>& b) {                    \
    for (int i = 0; i < N; ++i) if (!(a[i] == b[i])) return false;          \
    return true;                                                            \
  }                                                                         \
  template <typename T>                                                     \
  inline bool operator!=(const V<T>& a, const V<T>& b) { return !(a == b); }

SHIM_VEC_OPS(tvec2, 2)
SHIM_VEC_OPS(tvec3, 3)
SHIM_VEC_OPS(tvec4, 4)
#undef SHIM_VEC_OPS

using vec2 = tvec2<float>;
using vec3 = tvec3<float>;
using vec4 = tvec4<float>;
using dvec2 = tvec2<double>;
using dvec4 = tvec4<double>;
using uvec2 = tvec2<uint32_t>;
using ivec2 = tvec2<int32_t>;
using i32vec2 = tvec2<int32_t>;
using u64vec4 = tvec4<uint64_t>;

// ---- mat4 (column-major: m[c] is column c) --------------------------------
struct mat4 {
  vec4 c[4];
  mat4() : mat4(1.f) {}
  explicit mat4(float d) {
    for (int i = 0; i < 4; ++i) c[i] = vec4(0.f);
    c[0].x = d; c[1].y = d; c[2].z = d; c[3].w = d;
  }
  mat4(const vec4& a, const vec4& b, const vec4& cc, const vec4& d) {
    c[0] = a; c[1] = b; c[2] = cc; c[3] = d;
  }
  vec4& operator[](int i) { return c[i]; }
  const vec4& operator[](int i) const { return c[i]; }
};

inline vec4 operator*(const mat4& m, const vec4& v) {
  vec4 a0 = m[0] * v.x;
  vec4 a1 = m[1] * v.y;
  vec4 s0 = a0 + a1;
  vec4 a2 = m[2] * v.z;
  vec4 a3 = m[3] * v.w;
  vec4 s1 = a2 + a3;
  return s0 + s1;
}

inline mat4 operator*(const mat4& a, const mat4& b) {
  mat4 r(0.f);
  for (int j = 0; j < 4; ++j) {
    r[j] = a[0] * b[j].x + a[1] * b[j].y + a[2] * b[j].z + a[3] * b[j].w;
  }
  return r;
}

// ---- scalar helpers --------------------------------------------------------
template <typename T>
inline T floor(T v) { return std::floor(v); }
template <typename T>
inline T fract(T v) { return v - std::floor(v); }
template <typename T>
inline T clamp(T v, T lo, T hi) { return std::min(std::max(v, lo), hi); }
template <typename T>
inline T abs(T v) { return v < T(0) ? -v : v; }
inline float sqrt(float v) { return std::sqrt(v); }
inline double sqrt(double v) { return std::sqrt(v); }
template <typename T>
inline bool isinf(T v) { return std::isinf(v); }
template <typename T>
inline T min(T a, T b) { return b < a ? b : a; }
template <typename T>
inline T max(T a, T b) { return a < b ? b : a; }
// glm::mod is x - y * floor(x / y)
template <typename T>
inline T mod(T x, T y) { return x - y * std::floor(x / y); }
inline float cos(float v) { return std::cos(v); }
inline float sin(float v) { return std::sin(v); }
template <typename T>
constexpr T pi() { return static_cast<T>(3.14159265358979323846264338327950288); }
template <typename T>
constexpr T epsilon() { return std::numeric_limits<T>::epsilon(); }
template <typename T>
inline T radians(T deg) { return deg * static_cast<T>(0.01745329251994329576923690768489); }

template <typename T>
inline T dot(const tvec2<T>& a, const tvec2<T>& b) { return a.x * b.x + a.y * b.y; }
template <typename T>
inline T dot(const tvec3<T>& a, const tvec3<T>& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
inline T dot(const tvec4<T>& a, const tvec4<T>& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}
template <typename V>
inline V normalize(const V& v) {
  return v * (decltype(v.x))(1) / std::sqrt(dot(v, v));
}
inline float length(const vec2& v) { return std::sqrt(dot(v, v)); }

// ---- mat4 algebra ------------------------------------------------------------
inline float determinant(const mat4& m) {
  // cofactor expansion along the first column of the column-major matrix
  float s[6], t[6];
  s[0] = m[2][2] * m[3][3] - m[3][2] * m[2][3];
  s[1] = m[2][1] * m[3][3] - m[3][1] * m[2][3];
  s[2] = m[2][1] * m[3][2] - m[3][1] * m[2][2];
  s[3] = m[2][0] * m[3][3] - m[3][0] * m[2][3];
  s[4] = m[2][0] * m[3][2] - m[3][0] * m[2][2];
  s[5] = m[2][0] * m[3][1] - m[3][0] * m[2][1];
  t[0] = +(m[1][1] * s[0] - m[1][2] * s[1] + m[1][3] * s[2]);
  t[1] = -(m[1][0] * s[0] - m[1][2] * s[3] + m[1][3] * s[4]);
  t[2] = +(m[1][0] * s[1] - m[1][1] * s[3] + m[1][3] * s[5]);
  t[3] = -(m[1][0] * s[2] - m[1][1] * s[4] + m[1][2] * s[5]);
  (void)t;
  return m[0][0] * t[0] + m[0][1] * t[1] + m[0][2] * t[2] + m[0][3] * t[3];
}

inline mat4 inverse(const mat4& m) {
  // adjugate / determinant, computed with 2x2 sub-determinants
  float a[16];
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) a[c * 4 + r] = m[c][r];
  float inv[16];
  inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] +
           a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
  inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] -
           a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
  inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] +
           a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
  inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] -
            a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
  inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] -
           a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
  inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] +
           a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
  inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] -
           a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
  inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] +
            a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
  inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] +
           a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
  inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] -
           a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
  inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] +
            a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
  inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] -
            a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
  inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] -
           a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
  inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] +
           a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
  inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] -
            a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
  inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] +
            a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
  float det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
  float rdet = 1.0f / det;
  mat4 r(0.f);
  for (int c = 0; c < 4; ++c)
    for (int rr = 0; rr < 4; ++rr) r[c][rr] = inv[c * 4 + rr] * rdet;
  return r;
}

inline mat4 rotate(const mat4& m, float angle, const vec3& axis) {
  float c = std::cos(angle), s = std::sin(angle);
  float len = std::sqrt(dot(axis, axis));
  vec3 ax(axis.x / len, axis.y / len, axis.z / len);
  vec3 tmp(ax.x * (1 - c), ax.y * (1 - c), ax.z * (1 - c));
  mat4 rot(0.f);
  rot[0][0] = c + tmp.x * ax.x;
  rot[0][1] = tmp.x * ax.y + s * ax.z;
  rot[0][2] = tmp.x * ax.z - s * ax.y;
  rot[1][0] = tmp.y * ax.x - s * ax.z;
  rot[1][1] = c + tmp.y * ax.y;
  rot[1][2] = tmp.y * ax.z + s * ax.x;
  rot[2][0] = tmp.z * ax.x + s * ax.y;
  rot[2][1] = tmp.z * ax.y - s * ax.x;
  rot[2][2] = c + tmp.z * ax.z;
  mat4 r(0.f);
  r[0] = m[0] * rot[0][0] + m[1] * rot[0][1] + m[2] * rot[0][2];
  r[1] = m[0] * rot[1][0] + m[1] * rot[1][1] + m[2] * rot[1][2];
  r[2] = m[0] * rot[2][0] + m[1] * rot[2][1] + m[2] * rot[2][2];
  r[3] = m[3];
  return r;
}

inline bool isIdentity(const mat4& m, float eps) {
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) {
      float want = (c == r) ? 1.f : 0.f;
      // glm::epsilonEqual semantics: equal iff |a - b| < eps
      if (!(std::fabs(m[c][r] - want) < eps)) return false;
    }
  return true;
}

}  // namespace glm

#endif  // ORACLE_GLM_SHIM_GLM_HPP
