// Minimal stand-in for Granite's muglm vector types, enough for the reference's
// shared CPU/GPU headers (data_structures.h, swizzle_utils.h) to compile.
#pragma once
#include <stdint.h>
typedef uint32_t uint;
namespace muglm
{
template <typename T, int N> struct tvec { T v[N]; };
using ivec2 = tvec<int32_t, 2>;
using ivec3 = tvec<int32_t, 3>;
using ivec4 = tvec<int32_t, 4>;
using uvec2 = tvec<uint32_t, 2>;
using uvec3 = tvec<uint32_t, 3>;
using uvec4 = tvec<uint32_t, 4>;
using vec2 = tvec<float, 2>;
using vec3 = tvec<float, 3>;
using vec4 = tvec<float, 4>;
using u16vec2 = tvec<uint16_t, 2>;
using i16vec4 = tvec<int16_t, 4>;
}
