// BSDF value with derivatives (dual numbers) for the path-replay adjoint.
//
// The adjoint differentiates the closure value f(wo, wi) of the default
// (corrected) sampling mode with respect to base colour, roughness, metallic
// and specular, holding sampled directions, pdfs and MIS weights fixed
// (detached sampling, Vicini, Speierer, Jakob, "Path Replay Backpropagation",
// SIGGRAPH 2021). Each lobe follows the value half of the device closures in
// tr_bsdf.cuh (Disney.h:143-367, Microfacet.h:33-226, Diffuse.h:8-31).
#pragma once

#include "tr_bsdf.cuh"
#include "tr_dual.h"

namespace tr {
namespace dual {

struct Mat {
    Vec3<Dual> diffuse;
    Vec3<Dual> tint;
    Dual metallic;
    Dual specular;
    Dual roughness;
    float subsurface, specularTint, anisotropic, sheen, sheenTint, clearcoat, clearcoatGloss;
};

// material with the six parameters as independent variables; tint from CIE XYZ
// of the base colour (CudaMaterial.h:155-160, CudaUtility.h:32-50)
__device__ __forceinline__ Mat make(const HitMat& h)
{
    Mat m;
    m.diffuse = vec3(dvar(h.diffuse.x, kGBaseR), dvar(h.diffuse.y, kGBaseG), dvar(h.diffuse.z, kGBaseB));
    const Dual& r = m.diffuse.x;
    const Dual& g = m.diffuse.y;
    const Dual& b = m.diffuse.z;
    const Dual X = dmax(0.0f, 0.412453f * r + 0.357580f * g + 0.180423f * b);
    const Dual Y = dmax(0.0f, 0.212671f * r + 0.715160f * g + 0.072169f * b);
    const Dual Z = dmax(0.0f, 0.019334f * r + 0.119193f * g + 0.950227f * b);
    if (Y.v > 0.f) {
        const Dual iy = 1.f / Y;
        const Dual x = X * iy, y = Y * iy, z = Z * iy;
        m.tint = vec3(dmax(0.0f, 3.240479f * x - 1.537150f * y - 0.498535f * z),
                      dmax(0.0f, -0.969256f * x + 1.875992f * y + 0.041556f * z),
                      dmax(0.0f, 0.055648f * x - 0.204043f * y + 1.057311f * z));
    } else {
        m.tint = vec3(dconst(1.f), dconst(1.f), dconst(1.f));
    }
    m.roughness = dvar(h.roughness, kGRough);
    m.metallic = dvar(h.metallic, kGMetal);
    m.specular = dvar(h.specular, kGSpec);
    m.subsurface = h.subsurface;
    m.specularTint = h.specularTint;
    m.anisotropic = h.anisotropic;
    m.sheen = h.sheen;
    m.sheenTint = h.sheenTint;
    m.clearcoat = h.clearcoat;
    m.clearcoatGloss = h.clearcoatGloss;
    return m;
}

__device__ __forceinline__ Vec3<Dual> zero3() { return vec3(dconst(0.f), dconst(0.f), dconst(0.f)); }

__device__ __forceinline__ Vec3<Dual> diffuse_value(const Mat& m, const float3& wo, const float3& wi)
{
    const float3 h = normalize(wi + wo);
    const float con = wo.z, cin = wi.z, cih = dot(wi, h);
    const float fl = disney::schlick(cin), fv = disney::schlick(con);
    Dual fd = dconst(0.f);
    if (m.subsurface != 1.0f) {
        const Dual fd90 = 0.5f + (2.0f * square(cih)) * m.roughness;
        fd = ((1.f - fl) + fd90 * fl) * ((1.f - fv) + fd90 * fv);
    }
    if (m.subsurface > 0.0f) {
        const Dual fss90 = square(cih) * m.roughness;
        const Dual fss = ((1.f - fl) + fss90 * fl) * ((1.f - fv) + fss90 * fv);
        const Dual ss = 1.25f * (fss * (1.0f / (fabsf(con) + fabsf(cin)) - 0.5f) + 0.5f);
        fd = fd * (1.f - m.subsurface) + ss * m.subsurface;
    }
    const Dual k = fd * kRcpPi * (1.0f - m.metallic);
    return m.diffuse * k;
}

__device__ __forceinline__ Vec3<Dual> sheen_value(const Mat& m, const float3& wo, const float3& wi)
{
    const float3 h = normalize(wi + wo);
    const float fh = disney::schlick(dot(wi, h));
    const Vec3<Dual> t = vec3((1.f - m.sheenTint) + m.sheenTint * m.tint.x, (1.f - m.sheenTint) + m.sheenTint * m.tint.y,
                              (1.f - m.sheenTint) + m.sheenTint * m.tint.z);
    return t * ((fh * m.sheen) * (1.0f - m.metallic));
}

__device__ __forceinline__ Vec3<Dual> spec_fresnel(const Mat& m, const float3& o, const float3& h)
{
    const float st = m.specularTint;
    const Dual s = m.specular * 0.08f;
    Vec3<Dual> v = vec3(((1.f - st) + st * m.tint.x) * s, ((1.f - st) + st * m.tint.y) * s,
                        ((1.f - st) + st * m.tint.z) * s);
    const Dual om = 1.f - m.metallic;
    v = vec3(om * v.x + m.metallic * m.diffuse.x, om * v.y + m.metallic * m.diffuse.y,
             om * v.z + m.metallic * m.diffuse.z);
    const float f = disney::schlick(fabsf(dot(o, h)));
    return vec3((1.f - f) * v.x + f, (1.f - f) * v.y + f, (1.f - f) * v.z + f);
}

__device__ __forceinline__ void alpha_xy(const Mat& m, Dual& ax, Dual& ay)
{
    const Dual r2 = m.roughness * m.roughness;
    const float aspect = sqrtf(1.0f + m.anisotropic * (m.anisotropic < 0 ? 0.9f : -0.9f));
    ax = dmax(0.001f, r2 / aspect);
    ay = dmax(0.001f, r2 * aspect);
}

__device__ __forceinline__ Dual ggx_lambda(const float3& v, const Dual& ax, const Dual& ay)
{
    const float c = v.z;
    if (c == 0.0f)
        return dconst(0.f);
    const float c2 = square(c);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c2));
    Dual a;
    if (ax.v == ay.v || s == 0.0f) {
        a = ax;
    } else {
        const Dual px = (v.x / s) * ax, py = (v.y / s) * ay;
        a = dsqrt(px * px + py * py);
    }
    const float t2 = square(s) / c2;
    return (dsqrt(1.0f + (a * a) * t2) - 1.0f) * 0.5f;
}

__device__ __forceinline__ Dual ggx_D(const float3& m, const Dual& ax, const Dual& ay)
{
    const float c = m.z;
    if (c == 0.0f)
        return (ax * ax) * kRcpPi;
    const float c2 = square(c);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c2));
    const float c4 = square(c2);
    const float t2 = (1.0f - c2) / c2;
    Dual A;
    if (ax.v == ay.v || s == 0.0f) {
        A = 1.0f / (ax * ax);
    } else {
        const Dual qx = (m.x / s) / ax, qz = (m.z / s) / ay;
        A = qx * qx + qz * qz;
    }
    const Dual tmp = 1.0f + t2 * A;
    return 1.0f / ((kPi * c4) * (ax * ay) * (tmp * tmp));
}

__device__ __forceinline__ Vec3<Dual> ggx_value(const Mat& m, const float3& wo, const float3& wi)
{
    if (wo.z == 0.0f || wi.z == 0.0f)
        return zero3();
    const float3 h = normalize(wi + wo);
    if (dot(wo, h) == 0.0f)
        return zero3();
    Dual ax, ay;
    alpha_xy(m, ax, ay);
    const Dual D = ggx_D(h, ax, ay);
    const Dual G = 1.0f / (1.0f + ggx_lambda(wo, ax, ay) + ggx_lambda(wi, ax, ay));
    const Dual k = D * G * (1.0f / fabsf(4.0f * wo.z * wi.z));
    const Vec3<Dual> F = spec_fresnel(m, wo, h);
    return vec3(F.x * k, F.y * k, F.z * k);
}

// The full closure value of the default mode at (wo, wi): the sum of the lobes
// with a positive weight (disney::evaluate<false>), or diffuse / pi. The
// clearcoat lobe depends on no differentiated parameter and enters as a constant.
__device__ __forceinline__ Vec3<Dual> closure_value(uint32_t closure, const HitMat& hm, const float3& wo,
                                                    const float3& wi)
{
    const Mat m = make(hm);
    if (closure == TR_CLOSURE_DIFFUSE)
        return m.diffuse * kRcpPi;
    if (closure != TR_CLOSURE_DISNEY)
        return zero3();
    float wd, ws, wsp, wc;
    if (!disney::weights(hm, wd, ws, wsp, wc))
        return zero3();
    Vec3<Dual> f = zero3();
    if (wd > 0)
        f = f + diffuse_value(m, wo, wi);
    if (ws > 0)
        f = f + sheen_value(m, wo, wi);
    if (wsp > 0)
        f = f + ggx_value(m, wo, wi);
    if (wc > 0) {
        float3 v = f3(0.f);
        disney::gtr1_eval(disney::clearcoat_alpha(hm), hm, wo, wi, v);
        f = f + vec3(dconst(v.x), dconst(v.y), dconst(v.z));
    }
    return f;
}

} // namespace dual
} // namespace tr
