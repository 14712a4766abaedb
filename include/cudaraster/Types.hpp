// Types.hpp -- the framework's scalar and small vector types, shared by host
// code (CudaRaster.hpp, compiled by any C++17 compiler) and device code
// (PixelPipe.hpp, compiled by nvcc).
//
// Same names as the reference's framework (src/framework/base/Defs.hpp:40-55
// for S8..F64, src/framework/base/Math.hpp for Vec2i/Vec3i/Vec2f/Vec3f/
// Vec4f); only the members the host API and the pixel pipes use are here.
// The device arithmetic operators live in PixelPipe.hpp.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define CR_HOST_DEVICE __host__ __device__
#else
#define CR_HOST_DEVICE
#endif

namespace FW {

typedef int8_t S8;
typedef uint8_t U8;
typedef int16_t S16;
typedef uint16_t U16;
typedef int32_t S32;
typedef uint32_t U32;
typedef int64_t S64;
typedef uint64_t U64;
typedef float F32;
typedef double F64;

struct Vec2i {
    S32 x, y;
    CR_HOST_DEVICE Vec2i() : x(0), y(0) {}
    CR_HOST_DEVICE Vec2i(S32 a, S32 b) : x(a), y(b) {}
    CR_HOST_DEVICE bool operator==(const Vec2i& o) const { return x == o.x && y == o.y; }
    CR_HOST_DEVICE bool operator!=(const Vec2i& o) const { return !(*this == o); }
};
struct Vec3i {
    S32 x, y, z;
    CR_HOST_DEVICE Vec3i() : x(0), y(0), z(0) {}
    CR_HOST_DEVICE Vec3i(S32 a, S32 b, S32 c) : x(a), y(b), z(c) {}
    CR_HOST_DEVICE S32& operator[](int i) { return (&x)[i]; }
    CR_HOST_DEVICE const S32& operator[](int i) const { return (&x)[i]; }
};
struct Vec2f {
    F32 x, y;
    CR_HOST_DEVICE Vec2f() : x(0), y(0) {}
    CR_HOST_DEVICE Vec2f(F32 a) : x(a), y(a) {}
    CR_HOST_DEVICE Vec2f(F32 a, F32 b) : x(a), y(b) {}
};
struct Vec3f {
    F32 x, y, z;
    CR_HOST_DEVICE Vec3f() : x(0), y(0), z(0) {}
    CR_HOST_DEVICE Vec3f(F32 a) : x(a), y(a), z(a) {}
    CR_HOST_DEVICE Vec3f(F32 a, F32 b, F32 c) : x(a), y(b), z(c) {}
    CR_HOST_DEVICE F32& operator[](int i) { return (&x)[i]; }
    CR_HOST_DEVICE const F32& operator[](int i) const { return (&x)[i]; }
};
struct Vec4f {
    F32 x, y, z, w;
    CR_HOST_DEVICE Vec4f() : x(0), y(0), z(0), w(0) {}
    CR_HOST_DEVICE Vec4f(F32 a) : x(a), y(a), z(a), w(a) {}
    CR_HOST_DEVICE Vec4f(F32 a, F32 b, F32 c, F32 d) : x(a), y(b), z(c), w(d) {}
    CR_HOST_DEVICE Vec4f(const Vec3f& v, F32 d) : x(v.x), y(v.y), z(v.z), w(d) {}
    CR_HOST_DEVICE F32& operator[](int i) { return (&x)[i]; }
    CR_HOST_DEVICE const F32& operator[](int i) const { return (&x)[i]; }
};

}  // namespace FW
