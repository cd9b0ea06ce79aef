// Oracle test infrastructure -- not part of the shipped library.
//
// Minimal stand-in for the glm vector header that the reference includes as
// <glm/glm.hpp> (include/geometry.h:4). The reference's glm submodule
// (lib/glm, .gitmodules:1-3) is empty and pins no version, so this header
// restates only the documented glm vector semantics that the reference uses:
//   * vec<2|3|4, float> with x/y/z/w members and operator[];
//   * component-wise + - * / between vectors and with scalars (scalar
//     division divides each component, it does not multiply by a reciprocal);
//   * dot(a, b) = ((a.x*b.x + a.y*b.y) + a.z*b.z), left to right;
//   * cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y);
//   * length(v) = sqrt(dot(v, v)); normalize(v) = v * (1 / sqrt(dot(v, v)));
//   * mix(x, y, a) = x * (1 - a) + y * a; min/max/pow component-wise.
// Parity at this boundary is defined by this header (glm itself is absent).
// It deliberately includes <cmath> only (not <math.h>), as real glm does, so
// unqualified abs()/sqrt() overload resolution in the reference's TUs is the
// one their own include chains give.
#pragma once
#include <cmath>
#include <cstddef>
#include <algorithm>
#include <type_traits>

namespace glm {

enum qualifier { defaultp = 0 };

template <int L, typename T, qualifier Q = defaultp> struct vec;

template <typename T, qualifier Q> struct vec<2, T, Q> {
  T x, y;
  vec() = default;
  template <typename S, typename = std::enable_if_t<std::is_arithmetic<S>::value>>
  constexpr explicit vec(S s) : x(static_cast<T>(s)), y(static_cast<T>(s)) {}
  template <typename A, typename B>
  constexpr vec(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
  template <typename U, qualifier P>
  constexpr explicit vec(const vec<3, U, P>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)) {}
  T& operator[](int i) { return i == 0 ? x : y; }
  const T& operator[](int i) const { return i == 0 ? x : y; }
};

template <typename T, qualifier Q> struct vec<3, T, Q> {
  T x, y, z;
  vec() = default;
  template <typename S, typename = std::enable_if_t<std::is_arithmetic<S>::value>>
  constexpr explicit vec(S s) : x(static_cast<T>(s)), y(static_cast<T>(s)), z(static_cast<T>(s)) {}
  template <typename A, typename B, typename C>
  constexpr vec(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
  template <typename U, qualifier P>
  constexpr vec(const vec<4, U, P>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <typename T, qualifier Q> struct vec<4, T, Q> {
  T x, y, z, w;
  vec() = default;
  template <typename S, typename = std::enable_if_t<std::is_arithmetic<S>::value>>
  constexpr explicit vec(S s) : x(static_cast<T>(s)), y(static_cast<T>(s)), z(static_cast<T>(s)), w(static_cast<T>(s)) {}
  template <typename A, typename B, typename C, typename D>
  constexpr vec(A a, B b, C c, D d)
      : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)), w(static_cast<T>(d)) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

// ---- component-wise helpers -------------------------------------------------
template <int L, typename T, qualifier Q, typename F>
inline vec<L, T, Q> cw(const vec<L, T, Q>& a, const vec<L, T, Q>& b, F f) {
  vec<L, T, Q> r;
  for (int i = 0; i < L; ++i) r[i] = f(a[i], b[i]);
  return r;
}
template <int L, typename T, qualifier Q, typename F>
inline vec<L, T, Q> cws(const vec<L, T, Q>& a, T s, F f) {
  vec<L, T, Q> r;
  for (int i = 0; i < L; ++i) r[i] = f(a[i], s);
  return r;
}

#define GLMSHIM_BINOP(OP)                                                                  \
  template <int L, typename T, qualifier Q>                                                \
  inline vec<L, T, Q> operator OP(const vec<L, T, Q>& a, const vec<L, T, Q>& b) {          \
    return cw(a, b, [](T p, T q) { return p OP q; });                                      \
  }                                                                                        \
  template <int L, typename T, qualifier Q, typename S,                                     \
            typename = std::enable_if_t<std::is_arithmetic<S>::value>>                     \
  inline vec<L, T, Q> operator OP(const vec<L, T, Q>& a, S s) {                            \
    return cws(a, static_cast<T>(s), [](T p, T q) { return p OP q; });                     \
  }                                                                                        \
  template <int L, typename T, qualifier Q, typename S,                                     \
            typename = std::enable_if_t<std::is_arithmetic<S>::value>>                     \
  inline vec<L, T, Q> operator OP(S s, const vec<L, T, Q>& a) {                            \
    vec<L, T, Q> r;                                                                        \
    for (int i = 0; i < L; ++i) r[i] = static_cast<T>(s) OP a[i];                          \
    return r;                                                                              \
  }                                                                                        \
  template <int L, typename T, qualifier Q>                                                \
  inline vec<L, T, Q>& operator OP##=(vec<L, T, Q>& a, const vec<L, T, Q>& b) {            \
    a = a OP b;                                                                            \
    return a;                                                                              \
  }                                                                                        \
  template <int L, typename T, qualifier Q, typename S,                                     \
            typename = std::enable_if_t<std::is_arithmetic<S>::value>>                     \
  inline vec<L, T, Q>& operator OP##=(vec<L, T, Q>& a, S s) {                              \
    a = a OP static_cast<T>(s);                                                            \
    return a;                                                                              \
  }

GLMSHIM_BINOP(+)
GLMSHIM_BINOP(-)
GLMSHIM_BINOP(*)
GLMSHIM_BINOP(/)
#undef GLMSHIM_BINOP

template <int L, typename T, qualifier Q>
inline vec<L, T, Q> operator-(const vec<L, T, Q>& a) {
  vec<L, T, Q> r;
  for (int i = 0; i < L; ++i) r[i] = -a[i];
  return r;
}

// ---- geometric functions ----------------------------------------------------
template <typename T, qualifier Q>
inline T dot(const vec<2, T, Q>& a, const vec<2, T, Q>& b) { return a.x * b.x + a.y * b.y; }
template <typename T, qualifier Q>
inline T dot(const vec<3, T, Q>& a, const vec<3, T, Q>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T, qualifier Q>
inline T dot(const vec<4, T, Q>& a, const vec<4, T, Q>& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}
template <typename T, qualifier Q>
inline vec<3, T, Q> cross(const vec<3, T, Q>& a, const vec<3, T, Q>& b) {
  return vec<3, T, Q>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <int L, typename T, qualifier Q>
inline T length(const vec<L, T, Q>& v) { return std::sqrt(dot(v, v)); }
template <int L, typename T, qualifier Q>
inline vec<L, T, Q> normalize(const vec<L, T, Q>& v) {
  T inv = static_cast<T>(1) / std::sqrt(dot(v, v));
  return v * inv;
}

// ---- common functions --------------------------------------------------------
template <int L, typename T, qualifier Q>
inline vec<L, T, Q> min(const vec<L, T, Q>& a, const vec<L, T, Q>& b) {
  return cw(a, b, [](T p, T q) { return q < p ? q : p; });
}
template <int L, typename T, qualifier Q>
inline vec<L, T, Q> max(const vec<L, T, Q>& a, const vec<L, T, Q>& b) {
  return cw(a, b, [](T p, T q) { return p < q ? q : p; });
}
template <int L, typename T, qualifier Q>
inline vec<L, T, Q> min(const vec<L, T, Q>& a, T s) { return min(a, vec<L, T, Q>(s)); }
template <int L, typename T, qualifier Q>
inline vec<L, T, Q> max(const vec<L, T, Q>& a, T s) { return max(a, vec<L, T, Q>(s)); }
template <int L, typename T, qualifier Q>
inline vec<L, T, Q> pow(const vec<L, T, Q>& a, const vec<L, T, Q>& b) {
  return cw(a, b, [](T p, T q) { return std::pow(p, q); });
}
template <int L, typename T, qualifier Q>
inline vec<L, T, Q> mix(const vec<L, T, Q>& x, const vec<L, T, Q>& y, T a) {
  return x * (static_cast<T>(1) - a) + y * a;
}

using vec2 = vec<2, float>;
using vec3 = vec<3, float>;
using vec4 = vec<4, float>;

}  // namespace glm
