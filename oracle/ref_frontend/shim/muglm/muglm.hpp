// TEST INFRASTRUCTURE ONLY.  Stand-in for Granite's muglm vector library, enough
// for the reference's CPU frontend (gs/gs_interface.cpp, gs/gs_util.cpp) and its
// shared headers to compile here.  Written for this harness: component-wise
// vectors with x/y/z/w members, broadcast and converting constructors, the
// arithmetic / shift / bit operators the frontend uses, min/max/clamp/abs and
// the few swizzles it calls.
#pragma once
#include <stdint.h>
#include <cmath>
#include <algorithm>
typedef uint32_t uint;

namespace muglm
{
template <typename T> struct tvec2;
template <typename T> struct tvec3;
template <typename T> struct tvec4;

template <typename T>
struct tvec2
{
	T x, y;
	tvec2() = default;
	explicit tvec2(T s) : x(s), y(s) {}
	tvec2(T x_, T y_) : x(x_), y(y_) {}
	template <typename U> explicit tvec2(const tvec2<U> &o) : x(T(o.x)), y(T(o.y)) {}
	T &operator[](int i) { return (&x)[i]; }
	const T &operator[](int i) const { return (&x)[i]; }
	tvec4<T> xyxy() const { return tvec4<T>(x, y, x, y); }
	tvec2<T> yx() const { return tvec2<T>(y, x); }
};

template <typename T>
struct tvec3
{
	T x, y, z;
	tvec3() = default;
	explicit tvec3(T s) : x(s), y(s), z(s) {}
	tvec3(T x_, T y_, T z_) : x(x_), y(y_), z(z_) {}
	tvec3(const tvec2<T> &a, T z_) : x(a.x), y(a.y), z(z_) {}
	template <typename U> explicit tvec3(const tvec3<U> &o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
	T &operator[](int i) { return (&x)[i]; }
	const T &operator[](int i) const { return (&x)[i]; }
	tvec2<T> xy() const { return tvec2<T>(x, y); }
};

template <typename T>
struct tvec4
{
	T x, y, z, w;
	tvec4() = default;
	explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
	tvec4(T x_, T y_, T z_, T w_) : x(x_), y(y_), z(z_), w(w_) {}
	tvec4(const tvec2<T> &a, const tvec2<T> &b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
	tvec4(const tvec3<T> &a, T w_) : x(a.x), y(a.y), z(a.z), w(w_) {}
	template <typename U> explicit tvec4(const tvec4<U> &o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
	T &operator[](int i) { return (&x)[i]; }
	const T &operator[](int i) const { return (&x)[i]; }
	tvec2<T> xy() const { return tvec2<T>(x, y); }
	tvec2<T> zw() const { return tvec2<T>(z, w); }
	tvec2<T> xz() const { return tvec2<T>(x, z); }
	tvec2<T> yw() const { return tvec2<T>(y, w); }
	tvec3<T> xyz() const { return tvec3<T>(x, y, z); }
};

#define PGS_SHIM_VEC_BINOP(op)                                                                              \
	template <typename T> tvec2<T> operator op(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<T>(a.x op b.x, a.y op b.y); } \
	template <typename T> tvec3<T> operator op(const tvec3<T> &a, const tvec3<T> &b) { return tvec3<T>(a.x op b.x, a.y op b.y, a.z op b.z); } \
	template <typename T> tvec4<T> operator op(const tvec4<T> &a, const tvec4<T> &b) { return tvec4<T>(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w); } \
	template <typename T, typename S> tvec2<T> operator op(const tvec2<T> &a, S b) { return tvec2<T>(a.x op T(b), a.y op T(b)); } \
	template <typename T, typename S> tvec3<T> operator op(const tvec3<T> &a, S b) { return tvec3<T>(a.x op T(b), a.y op T(b), a.z op T(b)); } \
	template <typename T, typename S> tvec4<T> operator op(const tvec4<T> &a, S b) { return tvec4<T>(a.x op T(b), a.y op T(b), a.z op T(b), a.w op T(b)); } \
	template <typename T> tvec2<T> &operator op##=(tvec2<T> &a, const tvec2<T> &b) { a = a op b; return a; } \
	template <typename T> tvec3<T> &operator op##=(tvec3<T> &a, const tvec3<T> &b) { a = a op b; return a; } \
	template <typename T> tvec4<T> &operator op##=(tvec4<T> &a, const tvec4<T> &b) { a = a op b; return a; } \
	template <typename T, typename S> tvec2<T> &operator op##=(tvec2<T> &a, S b) { a = a op b; return a; } \
	template <typename T, typename S> tvec3<T> &operator op##=(tvec3<T> &a, S b) { a = a op b; return a; } \
	template <typename T, typename S> tvec4<T> &operator op##=(tvec4<T> &a, S b) { a = a op b; return a; }

PGS_SHIM_VEC_BINOP(+)
PGS_SHIM_VEC_BINOP(-)
PGS_SHIM_VEC_BINOP(*)
PGS_SHIM_VEC_BINOP(/)
PGS_SHIM_VEC_BINOP(>>)
PGS_SHIM_VEC_BINOP(<<)
PGS_SHIM_VEC_BINOP(&)
PGS_SHIM_VEC_BINOP(|)
#undef PGS_SHIM_VEC_BINOP

template <typename T> tvec2<T> operator-(const tvec2<T> &a) { return tvec2<T>(-a.x, -a.y); }
template <typename T> tvec4<T> operator-(const tvec4<T> &a) { return tvec4<T>(-a.x, -a.y, -a.z, -a.w); }
template <typename T> bool operator==(const tvec2<T> &a, const tvec2<T> &b) { return a.x == b.x && a.y == b.y; }
template <typename T> bool operator!=(const tvec2<T> &a, const tvec2<T> &b) { return !(a == b); }
template <typename T> bool operator==(const tvec4<T> &a, const tvec4<T> &b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }
template <typename T> bool operator!=(const tvec4<T> &a, const tvec4<T> &b) { return !(a == b); }

template <typename T> T min(T a, T b) { return b < a ? b : a; }
template <typename T> T max(T a, T b) { return a < b ? b : a; }
template <typename T> T clamp(T v, T lo, T hi) { return min(max(v, lo), hi); }
template <typename T> tvec2<T> min(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<T>(min(a.x, b.x), min(a.y, b.y)); }
template <typename T> tvec2<T> max(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<T>(max(a.x, b.x), max(a.y, b.y)); }
template <typename T> tvec3<T> min(const tvec3<T> &a, const tvec3<T> &b) { return tvec3<T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
template <typename T> tvec3<T> max(const tvec3<T> &a, const tvec3<T> &b) { return tvec3<T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
template <typename T> tvec4<T> min(const tvec4<T> &a, const tvec4<T> &b) { return tvec4<T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z), min(a.w, b.w)); }
template <typename T> tvec4<T> max(const tvec4<T> &a, const tvec4<T> &b) { return tvec4<T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
template <typename T> tvec2<T> clamp(const tvec2<T> &v, const tvec2<T> &lo, const tvec2<T> &hi) { return min(max(v, lo), hi); }
template <typename T> tvec4<T> clamp(const tvec4<T> &v, const tvec4<T> &lo, const tvec4<T> &hi) { return min(max(v, lo), hi); }
inline int abs(int v) { return v < 0 ? -v : v; }
inline float abs(float v) { return std::fabs(v); }
template <typename T> tvec2<T> abs(const tvec2<T> &a) { return tvec2<T>(abs(a.x), abs(a.y)); }
inline float floor(float v) { return std::floor(v); }
inline float ceil(float v) { return std::ceil(v); }

template <typename T> tvec2<bool> notEqual(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<bool>(a.x != b.x, a.y != b.y); }
template <typename T> tvec2<bool> equal(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<bool>(a.x == b.x, a.y == b.y); }
template <typename T> tvec2<bool> greaterThan(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<bool>(a.x > b.x, a.y > b.y); }
template <typename T> tvec2<bool> lessThan(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<bool>(a.x < b.x, a.y < b.y); }
template <typename T> tvec3<bool> notEqual(const tvec3<T> &a, const tvec3<T> &b) { return tvec3<bool>(a.x != b.x, a.y != b.y, a.z != b.z); }
template <typename T> tvec4<bool> notEqual(const tvec4<T> &a, const tvec4<T> &b) { return tvec4<bool>(a.x != b.x, a.y != b.y, a.z != b.z, a.w != b.w); }
inline bool any(const tvec2<bool> &v) { return v.x || v.y; }
inline bool all(const tvec2<bool> &v) { return v.x && v.y; }
inline bool any(const tvec3<bool> &v) { return v.x || v.y || v.z; }
inline bool all(const tvec3<bool> &v) { return v.x && v.y && v.z; }
inline bool any(const tvec4<bool> &v) { return v.x || v.y || v.z || v.w; }
inline bool all(const tvec4<bool> &v) { return v.x && v.y && v.z && v.w; }

using ivec2 = tvec2<int32_t>;
using ivec3 = tvec3<int32_t>;
using ivec4 = tvec4<int32_t>;
using uvec2 = tvec2<uint32_t>;
using uvec3 = tvec3<uint32_t>;
using uvec4 = tvec4<uint32_t>;
using vec2 = tvec2<float>;
using vec3 = tvec3<float>;
using vec4 = tvec4<float>;
using u16vec2 = tvec2<uint16_t>;
using i16vec2 = tvec2<int16_t>;
using i16vec4 = tvec4<int16_t>;
using u16vec4 = tvec4<uint16_t>;
using u8vec4 = tvec4<uint8_t>;
using bvec2 = tvec2<bool>;
}
