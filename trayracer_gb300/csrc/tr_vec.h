// Small float2/float3/float4 vector algebra shared by the host build code and
// the device kernels (the role helper_math.h and CudaLinearMath.h play in the
// reference, thirdparty/CUDA/helper_math.h, Tracer/CUDA/GPU/CudaLinearMath.h).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define TR_HD __host__ __device__ __forceinline__
#else
#define TR_HD inline
#endif

namespace tr {

constexpr float kPi = 3.1415926535897932f;
constexpr float kTwoPi = 6.2831853071795865f;
constexpr float kRcpPi = 0.3183098861837907f;
constexpr float kRcpTwoPi = 0.1591549430918953f;
constexpr float kPiOver2 = 1.57079632679f;
constexpr float kPiOver4 = 0.78539816339f;
// Epsilon of the shading code, Tracer/CUDA/GPU/CudaGlobals.h:10.
constexpr float kEpsilon = 1e-3f;
// Ray tmax of every closest-hit query, Tracer/Optix/GPU/optix.cu:16.
constexpr float kDstMax = 1e30f;

TR_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
TR_HD float3 f3(float s) { return make_float3(s, s, s); }
TR_HD float3 f3(const float4& v) { return make_float3(v.x, v.y, v.z); }
TR_HD float4 f4(const float3& v, float w) { return make_float4(v.x, v.y, v.z, w); }

TR_HD float3 operator+(const float3& a, const float3& b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
TR_HD float3 operator-(const float3& a, const float3& b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
TR_HD float3 operator*(const float3& a, const float3& b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
TR_HD float3 operator/(const float3& a, const float3& b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
TR_HD float3 operator*(const float3& a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
TR_HD float3 operator*(float s, const float3& a) { return make_float3(a.x * s, a.y * s, a.z * s); }
TR_HD float3 operator/(const float3& a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
TR_HD float3 operator+(const float3& a, float s) { return make_float3(a.x + s, a.y + s, a.z + s); }
TR_HD float3 operator+(float s, const float3& a) { return make_float3(a.x + s, a.y + s, a.z + s); }
TR_HD float3 operator-(const float3& a) { return make_float3(-a.x, -a.y, -a.z); }
TR_HD float3& operator+=(float3& a, const float3& b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
TR_HD float3& operator*=(float3& a, const float3& b) { a.x *= b.x; a.y *= b.y; a.z *= b.z; return a; }
TR_HD float3& operator*=(float3& a, float s) { a.x *= s; a.y *= s; a.z *= s; return a; }
TR_HD float2 operator+(const float2& a, const float2& b) { return make_float2(a.x + b.x, a.y + b.y); }
TR_HD float2 operator-(const float2& a, const float2& b) { return make_float2(a.x - b.x, a.y - b.y); }
TR_HD float2 operator*(const float2& a, float s) { return make_float2(a.x * s, a.y * s); }
TR_HD float2 operator*(float s, const float2& a) { return make_float2(a.x * s, a.y * s); }
TR_HD float4 operator+(const float4& a, const float4& b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }

TR_HD float dot(const float3& a, const float3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
TR_HD float3 cross(const float3& a, const float3& b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
TR_HD float length(const float3& v) { return sqrtf(dot(v, v)); }
TR_HD float rsqrt_(float x)
{
#if defined(__CUDA_ARCH__)
    return rsqrtf(x);
#else
    return 1.0f / sqrtf(x);
#endif
}
TR_HD float3 normalize(const float3& v) { return v * rsqrt_(dot(v, v)); }
// a / b for shading arithmetic: the device's fast division (within 2 ulp; the
// traversal keeps its correctly rounded operations), plain division on the host
TR_HD float fdiv(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fdividef(a, b);
#else
    return a / b;
#endif
}
TR_HD float2 normalize(const float2& v) { return v * rsqrt_(v.x * v.x + v.y * v.y); }
TR_HD float fminf_(float a, float b) { return a < b ? a : b; }
TR_HD float fmaxf_(float a, float b) { return a > b ? a : b; }
TR_HD float clampf(float x, float lo, float hi) { return fmaxf_(lo, fminf_(x, hi)); }
TR_HD float saturate(float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }
TR_HD float square(float x) { return x * x; }
TR_HD float mix(float a, float b, float t) { return (a * (1.f - t)) + (b * t); }
TR_HD float lerp(float a, float b, float t) { return a + t * (b - a); }
TR_HD float3 reflect(const float3& i, const float3& n) { return i - 2.0f * n * dot(n, i); }

TR_HD uint32_t f2u(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
TR_HD float u2f(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

// Colour helpers, Tracer/CUDA/GPU/CudaUtility.h:32-50.
TR_HD float3 linear_to_xyz(const float3& rgb)
{
    return make_float3(fmaxf_(0.0f, 0.412453f * rgb.x + 0.357580f * rgb.y + 0.180423f * rgb.z),
                       fmaxf_(0.0f, 0.212671f * rgb.x + 0.715160f * rgb.y + 0.072169f * rgb.z),
                       fmaxf_(0.0f, 0.019334f * rgb.x + 0.119193f * rgb.y + 0.950227f * rgb.z));
}
TR_HD float3 xyz_to_linear(const float3& xyz)
{
    return make_float3(fmaxf_(0.0f, 3.240479f * xyz.x - 1.537150f * xyz.y - 0.498535f * xyz.z),
                       fmaxf_(0.0f, -0.969256f * xyz.x + 1.875992f * xyz.y + 0.041556f * xyz.z),
                       fmaxf_(0.0f, 0.055648f * xyz.x - 0.204043f * xyz.y + 1.057311f * xyz.z));
}

} // namespace tr
