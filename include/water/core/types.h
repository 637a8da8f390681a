// Small POD types of the C++ façade. Same names and layouts as the reference's
// water/core/types.h (core/include/water/core/types.h:9-27) so that code written
// against the reference compiles unchanged: Vec3f is 12 bytes, AoS.
#pragma once

#include <cstdint>

namespace water {

using u8 = std::uint8_t;
using u16 = std::uint16_t;
using u32 = std::uint32_t;
using u64 = std::uint64_t;
using i8 = std::int8_t;
using i16 = std::int16_t;
using i32 = std::int32_t;
using i64 = std::int64_t;
using f32 = float;
using f64 = double;

struct Vec3f { f32 x, y, z; };
struct Vec3i { i32 x, y, z; };
struct Vec4f { f32 x, y, z, w; };
struct Vec3u { u32 x, y, z; };

inline constexpr Vec3f kZero3f{0.0f, 0.0f, 0.0f};

static_assert(sizeof(Vec3f) == 12, "Vec3f is three packed floats");

}  // namespace water
