// glsl_shim.h — just enough of GLSL's vector types and built-ins, in C++, to
// compile the reference's shaderio headers and a few of its shader files
// unchanged (after the mechanical rewrite of oracle/glsl_to_cpp.py).
//
// TEST INFRASTRUCTURE (oracle side): used only by oracle/ref_shader_pin.cpp,
// which pins the oracle's restatement to the reference's own code.
//
// The headers `using namespace glm;` (shaders/shaderio_core.h:28), so the
// types live in a namespace of that name; they are this file's own minimal
// definitions, not the glm library. Layout matches what the shaderio headers
// expect from glm's defaults: tightly packed floats / ints, 4-byte alignment
// for every float vector and matrix, mat4 as four column vec4s.
//
// Built-ins follow the GLSL 4.60 specification's definitions. Where the
// specification leaves the arithmetic open, the choice is stated:
//   - round(): ties to even (the specification lets an implementation pick);
//   - dot(): (x0*y0 + x1*y1) + x2*y2 [+ x3*y3], left to right, no contraction;
//   - length(x) = sqrt(dot(x, x)); distance(a, b) = length(a - b);
//   - normalize(x) = x / length(x) (the specification's formula);
//   - matrix products: each result component sums the column terms left to
//     right (m[0]*v.x + m[1]*v.y) + m[2]*v.z + m[3]*v.w;
//   - pow, sin, cos: the C library's float functions.
// The file is compiled with -ffp-contract=off, so no a*b+c is fused.
#pragma once

#include <cmath>
#include <cstdint>
#include <type_traits>

namespace glm {

typedef uint32_t uint;

template <class T>
struct tvec2;
template <class T>
struct tvec3;
template <class T>
struct tvec4;

template <class S>
using if_scalar = typename std::enable_if<std::is_arithmetic<S>::value, int>::type;

template <class T>
struct tvec2
{
  T x, y;
  tvec2() = default;
  template <class S, if_scalar<S> = 0>
  explicit tvec2(S s) : x(T(s)), y(T(s)) {}
  template <class A, class B>
  tvec2(A a, B b) : x(T(a)), y(T(b)) {}
  template <class U>
  explicit tvec2(const tvec2<U>& v) : x(T(v.x)), y(T(v.y)) {}
  T&       operator[](int i) { return (&x)[i]; }
  const T& operator[](int i) const { return (&x)[i]; }
  tvec2 xy() const { return *this; }
  tvec2 yx() const { return {y, x}; }
};

template <class T>
struct tvec3
{
  T x, y, z;
  tvec3() = default;
  template <class S, if_scalar<S> = 0>
  explicit tvec3(S s) : x(T(s)), y(T(s)), z(T(s)) {}
  template <class A, class B, class C>
  tvec3(A a, B b, C c) : x(T(a)), y(T(b)), z(T(c)) {}
  template <class U>
  explicit tvec3(const tvec3<U>& v) : x(T(v.x)), y(T(v.y)), z(T(v.z)) {}
  T&       operator[](int i) { return (&x)[i]; }
  const T& operator[](int i) const { return (&x)[i]; }
  tvec2<T> xy() const { return {x, y}; }
  tvec3    xyz() const { return *this; }
  tvec3    yzx() const { return {y, z, x}; }
  tvec3    zxy() const { return {z, x, y}; }
  tvec3    xzy() const { return {x, z, y}; }
  tvec3    yxz() const { return {y, x, z}; }
  tvec3    zyx() const { return {z, y, x}; }
};

template <class T>
struct tvec4
{
  T x, y, z, w;
  tvec4() = default;
  template <class S, if_scalar<S> = 0>
  explicit tvec4(S s) : x(T(s)), y(T(s)), z(T(s)), w(T(s)) {}
  template <class A, class B, class C, class D>
  tvec4(A a, B b, C c, D d) : x(T(a)), y(T(b)), z(T(c)), w(T(d)) {}
  template <class U, class S>
  tvec4(const tvec3<U>& v, S s) : x(T(v.x)), y(T(v.y)), z(T(v.z)), w(T(s)) {}
  template <class U, class V>
  tvec4(const tvec2<U>& a, const tvec2<V>& b) : x(T(a.x)), y(T(a.y)), z(T(b.x)), w(T(b.y)) {}
  template <class U>
  explicit tvec4(const tvec4<U>& v) : x(T(v.x)), y(T(v.y)), z(T(v.z)), w(T(v.w)) {}
  T&          operator[](int i) { return (&x)[i]; }
  const T&    operator[](int i) const { return (&x)[i]; }
  tvec2<T>    xy() const { return {x, y}; }
  tvec2<T>    zw() const { return {z, w}; }
  tvec3<T>    xyz() const { return {x, y, z}; }
  tvec4       xyzw() const { return *this; }
};

// component-wise arithmetic: vector op vector, vector op scalar, scalar op vector
#define GLSL_SHIM_OPS(OP)                                                                                              \
  template <class T>                                                                                                   \
  tvec2<T> operator OP(const tvec2<T>& a, const tvec2<T>& b)                                                           \
  {                                                                                                                    \
    return {T(a.x OP b.x), T(a.y OP b.y)};                                                                             \
  }                                                                                                                    \
  template <class T>                                                                                                   \
  tvec3<T> operator OP(const tvec3<T>& a, const tvec3<T>& b)                                                           \
  {                                                                                                                    \
    return {T(a.x OP b.x), T(a.y OP b.y), T(a.z OP b.z)};                                                              \
  }                                                                                                                    \
  template <class T>                                                                                                   \
  tvec4<T> operator OP(const tvec4<T>& a, const tvec4<T>& b)                                                           \
  {                                                                                                                    \
    return {T(a.x OP b.x), T(a.y OP b.y), T(a.z OP b.z), T(a.w OP b.w)};                                               \
  }                                                                                                                    \
  template <class T, class S, if_scalar<S> = 0>                                                                        \
  tvec2<T> operator OP(const tvec2<T>& a, S s)                                                                         \
  {                                                                                                                    \
    return {T(a.x OP T(s)), T(a.y OP T(s))};                                                                           \
  }                                                                                                                    \
  template <class T, class S, if_scalar<S> = 0>                                                                        \
  tvec3<T> operator OP(const tvec3<T>& a, S s)                                                                         \
  {                                                                                                                    \
    return {T(a.x OP T(s)), T(a.y OP T(s)), T(a.z OP T(s))};                                                           \
  }                                                                                                                    \
  template <class T, class S, if_scalar<S> = 0>                                                                        \
  tvec4<T> operator OP(const tvec4<T>& a, S s)                                                                         \
  {                                                                                                                    \
    return {T(a.x OP T(s)), T(a.y OP T(s)), T(a.z OP T(s)), T(a.w OP T(s))};                                           \
  }                                                                                                                    \
  template <class T, class S, if_scalar<S> = 0>                                                                        \
  tvec2<T> operator OP(S s, const tvec2<T>& a)                                                                         \
  {                                                                                                                    \
    return {T(T(s) OP a.x), T(T(s) OP a.y)};                                                                           \
  }                                                                                                                    \
  template <class T, class S, if_scalar<S> = 0>                                                                        \
  tvec3<T> operator OP(S s, const tvec3<T>& a)                                                                         \
  {                                                                                                                    \
    return {T(T(s) OP a.x), T(T(s) OP a.y), T(T(s) OP a.z)};                                                           \
  }                                                                                                                    \
  template <class T, class S, if_scalar<S> = 0>                                                                        \
  tvec4<T> operator OP(S s, const tvec4<T>& a)                                                                         \
  {                                                                                                                    \
    return {T(T(s) OP a.x), T(T(s) OP a.y), T(T(s) OP a.z), T(T(s) OP a.w)};                                           \
  }                                                                                                                    \
  template <class T, class R>                                                                                          \
  tvec3<T>& operator OP##=(tvec3<T>& a, const R& b)                                                                    \
  {                                                                                                                    \
    return a = a OP b;                                                                                                 \
  }                                                                                                                    \
  template <class T, class R>                                                                                          \
  tvec2<T>& operator OP##=(tvec2<T>& a, const R& b)                                                                    \
  {                                                                                                                    \
    return a = a OP b;                                                                                                 \
  }                                                                                                                    \
  template <class T, class R>                                                                                          \
  tvec4<T>& operator OP##=(tvec4<T>& a, const R& b)                                                                    \
  {                                                                                                                    \
    return a = a OP b;                                                                                                 \
  }

GLSL_SHIM_OPS(+)
GLSL_SHIM_OPS(-)
GLSL_SHIM_OPS(*)
GLSL_SHIM_OPS(/)
#undef GLSL_SHIM_OPS

template <class T>
tvec3<T> operator-(const tvec3<T>& a)
{
  return {-a.x, -a.y, -a.z};
}

typedef tvec2<float>    vec2;
typedef tvec3<float>    vec3;
typedef tvec4<float>    vec4;
typedef tvec2<int32_t>  ivec2;
typedef tvec3<int32_t>  ivec3;
typedef tvec4<int32_t>  ivec4;
typedef tvec2<uint32_t> uvec2;
typedef tvec3<uint32_t> uvec3;
typedef tvec4<uint32_t> uvec4;
typedef tvec3<uint8_t>  u8vec3;
typedef tvec4<uint8_t>  u8vec4;
typedef tvec2<bool>     bvec2;
typedef tvec3<bool>     bvec3;

// column-major 4x4 matrix (m[c] is column c)
struct mat4
{
  vec4        c[4];
  vec4&       operator[](int i) { return c[i]; }
  const vec4& operator[](int i) const { return c[i]; }
};

inline vec4 operator*(const mat4& m, const vec4& v)
{
  vec4 r;
  for(int i = 0; i < 4; i++)
    r[i] = ((m[0][i] * v.x + m[1][i] * v.y) + m[2][i] * v.z) + m[3][i] * v.w;
  return r;
}

inline mat4 operator*(const mat4& a, const mat4& b)
{
  mat4 r;
  for(int c = 0; c < 4; c++)
    r[c] = a * b[c];
  return r;
}

static_assert(sizeof(vec3) == 12 && alignof(vec3) == 4, "vec3 layout");
static_assert(sizeof(vec4) == 16 && alignof(vec4) == 4, "vec4 layout");
static_assert(sizeof(mat4) == 64 && alignof(mat4) == 4, "mat4 layout");
static_assert(sizeof(uvec3) == 12 && sizeof(ivec2) == 8 && sizeof(u8vec4) == 4, "integer vector layout");

// ---- built-ins (GLSL 4.60, chapter 8) ----------------------------------------

// min(x, y): y if y < x, else x; max(x, y): y if x < y, else x
template <class T, if_scalar<T> = 0>
T min(T x, T y)
{
  return y < x ? y : x;
}
template <class T, if_scalar<T> = 0>
T max(T x, T y)
{
  return x < y ? y : x;
}
template <class T>
tvec2<T> min(const tvec2<T>& a, const tvec2<T>& b)
{
  return {min(a.x, b.x), min(a.y, b.y)};
}
template <class T>
tvec3<T> min(const tvec3<T>& a, const tvec3<T>& b)
{
  return {min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)};
}
template <class T>
tvec4<T> min(const tvec4<T>& a, const tvec4<T>& b)
{
  return {min(a.x, b.x), min(a.y, b.y), min(a.z, b.z), min(a.w, b.w)};
}
template <class T>
tvec2<T> max(const tvec2<T>& a, const tvec2<T>& b)
{
  return {max(a.x, b.x), max(a.y, b.y)};
}
template <class T>
tvec3<T> max(const tvec3<T>& a, const tvec3<T>& b)
{
  return {max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)};
}
template <class T>
tvec4<T> max(const tvec4<T>& a, const tvec4<T>& b)
{
  return {max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)};
}
// clamp(x, lo, hi) = min(max(x, lo), hi)
template <class V>
V clamp(const V& x, const V& lo, const V& hi)
{
  return min(max(x, lo), hi);
}

inline float abs(float x) { return std::fabs(x); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float pow(float x, float y) { return std::pow(x, y); }

// round(): ties to even (nearbyint under the default rounding mode)
inline float round(float x) { return std::nearbyint(x); }
inline vec3  round(const vec3& v) { return {round(v.x), round(v.y), round(v.z)}; }

inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec3& v) { return sqrt(dot(v, v)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline vec3  normalize(const vec3& v) { return v / length(v); }

// mix(x, y, a) with a boolean selector: y where a is true, x elsewhere
inline vec3 mix(const vec3& x, const vec3& y, const bvec3& a) { return {a.x ? y.x : x.x, a.y ? y.y : x.y, a.z ? y.z : x.z}; }

inline bvec2 greaterThan(const vec2& a, const vec2& b) { return {a.x > b.x, a.y > b.y}; }
inline bool  any(const bvec2& v) { return v.x || v.y; }

// GL_EXT_shader_explicit_arithmetic_types: unpack8(uint) -> u8vec4, x = low byte
inline u8vec4 unpack8(uint32_t v)
{
  return {uint8_t(v & 0xFF), uint8_t((v >> 8) & 0xFF), uint8_t((v >> 16) & 0xFF), uint8_t(v >> 24)};
}

}  // namespace glm
