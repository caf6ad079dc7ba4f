// Forward-mode dual numbers for the adjoint: a value and its partial
// derivatives with respect to the six differentiated material parameters
// (base colour r, g, b, roughness, metallic, specular), host and device.
#pragma once

#include "tr_vec.h"

namespace tr {

constexpr int kGradParams = 6;          // base colour rgb, roughness, metallic, specular
constexpr int kGradSlots = 9;           // + emission rgb, per material
enum GradParam { kGBaseR = 0, kGBaseG, kGBaseB, kGRough, kGMetal, kGSpec, kGEmR, kGEmG, kGEmB };

struct Dual {
    float v;
    float d[kGradParams];
};

TR_HD Dual dconst(float v)
{
    Dual r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < kGradParams; ++i)
        r.d[i] = 0.f;
    return r;
}
TR_HD Dual dvar(float v, int k)
{
    Dual r = dconst(v);
    r.d[k] = 1.f;
    return r;
}
TR_HD Dual operator+(const Dual& a, const Dual& b)
{
    Dual r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < kGradParams; ++i)
        r.d[i] = a.d[i] + b.d[i];
    return r;
}
TR_HD Dual operator-(const Dual& a, const Dual& b)
{
    Dual r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < kGradParams; ++i)
        r.d[i] = a.d[i] - b.d[i];
    return r;
}
TR_HD Dual operator-(const Dual& a)
{
    Dual r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < kGradParams; ++i)
        r.d[i] = -a.d[i];
    return r;
}
TR_HD Dual operator*(const Dual& a, const Dual& b)
{
    Dual r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < kGradParams; ++i)
        r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
TR_HD Dual operator/(const Dual& a, const Dual& b)
{
    Dual r;
    const float inv = 1.f / b.v;
    r.v = a.v * inv;
#pragma unroll
    for (int i = 0; i < kGradParams; ++i)
        r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
    return r;
}
TR_HD Dual operator+(const Dual& a, float b) { Dual r = a; r.v += b; return r; }
TR_HD Dual operator+(float b, const Dual& a) { return a + b; }
TR_HD Dual operator-(const Dual& a, float b) { Dual r = a; r.v -= b; return r; }
TR_HD Dual operator-(float b, const Dual& a) { return dconst(b) - a; }
TR_HD Dual operator*(const Dual& a, float b)
{
    Dual r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < kGradParams; ++i)
        r.d[i] = a.d[i] * b;
    return r;
}
TR_HD Dual operator*(float b, const Dual& a) { return a * b; }
TR_HD Dual operator/(const Dual& a, float b) { return a * (1.f / b); }
TR_HD Dual operator/(float a, const Dual& b) { return dconst(a) / b; }
TR_HD Dual dsqrt(const Dual& a)
{
    Dual r;
    r.v = sqrtf(a.v);
    const float k = r.v > 0.f ? 0.5f / r.v : 0.f;
#pragma unroll
    for (int i = 0; i < kGradParams; ++i)
        r.d[i] = a.d[i] * k;
    return r;
}
TR_HD Dual dmax(const Dual& a, float b) { return a.v > b ? a : dconst(b); }
TR_HD Dual dmax(float b, const Dual& a) { return dmax(a, b); }
TR_HD bool operator<(const Dual& a, float b) { return a.v < b; }
TR_HD bool operator>(const Dual& a, float b) { return a.v > b; }

// three-component vectors over a scalar type (float or Dual)
template <class S>
struct Vec3 {
    S x, y, z;
};
template <class S> TR_HD Vec3<S> vec3(const S& x, const S& y, const S& z) { return Vec3<S>{x, y, z}; }
template <class S> TR_HD Vec3<S> operator+(const Vec3<S>& a, const Vec3<S>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class S> TR_HD Vec3<S> operator*(const Vec3<S>& a, const S& s) { return {a.x * s, a.y * s, a.z * s}; }
template <class S> TR_HD Vec3<S> operator*(const Vec3<S>& a, float s) { return {a.x * s, a.y * s, a.z * s}; }
template <class S> TR_HD Vec3<S> operator*(float s, const Vec3<S>& a) { return {a.x * s, a.y * s, a.z * s}; }
template <class S> TR_HD Vec3<S> operator+(const Vec3<S>& a, float s) { return {a.x + s, a.y + s, a.z + s}; }

} // namespace tr
