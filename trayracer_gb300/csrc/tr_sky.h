// Preetham sky model as the reference evaluates it (SampleSky,
// Tracer/CUDA/GPU/CudaSky.h:105-156; Preetham, Shirley, Smits, "A Practical
// Analytic Model for Daylight", SIGGRAPH 1999): the terms that depend only on
// the sky settings are computed once on the host (make_sky), the per-direction
// remainder on the device (sky_radiance) with the same operations in the same
// order.
#pragma once

#include <cmath>

#include "tr_device.h"

namespace tr {

namespace sky {
constexpr float kMieCoefficient = 0.005f;
constexpr float kMieG = 0.80f;
constexpr float kMieV = 4.f;
constexpr float kMieZenithLength = 1.25e3f;
constexpr float kRayleighCoefficient = 2.5f;
constexpr float kRayleighZenithLength = 8.4e3f;
constexpr float kDepolarization = 0.031f;
constexpr float kMolecules = 2.545e25f;
constexpr float kRefractiveIndex = 1.0003f;
constexpr float kSunFalloffSteepness = 1.5f;
}  // namespace sky

// Sky::Build + the direction-independent part of SampleSky (host).
inline SkyView make_sky(const tr_sky_desc& d)
{
    SkyView v{};
    // Sky::SetSunDir normalises, Sky::SetTurbidity clamps to [1, 10]
    const float len2 = d.sun_dir[0] * d.sun_dir[0] + d.sun_dir[1] * d.sun_dir[1] + d.sun_dir[2] * d.sun_dir[2];
    const float inv = 1.0f / std::sqrt(len2);
    v.sunDir = make_float3(d.sun_dir[0] * inv, d.sun_dir[1] * inv, d.sun_dir[2] * inv);
    const float turbidity = std::fmin(std::fmax(d.turbidity, 1.f), 10.f);
    v.enabled = d.enabled ? 1u : 0u;
    v.drawSun = d.draw_sun ? 1.f : 0.f;
    const float diameter = d.sun_angular_diameter * kPi / (60.f * 180.f);
    const float radius = diameter * .5f;
    v.sunArea = kPi * radius * radius;
    v.cosSunAngularDiameter = std::cos(diameter);
    v.sunEnergy = d.enabled ? d.sun_intensity * d.selection_bias : 0.f;

    const float cosSunUp = v.sunDir.y;  // dot(sunDir, (0, 1, 0))
    float sunfade = 1.f - std::fmin(std::fmax(1.f - std::exp(-v.sunDir.z / 500.f), 0.f), 1.f);
    const float rayleigh = sky::kRayleighCoefficient - (1.f * (1.f - sunfade));
    const float lambda[3] = {620e-9f, 492e-9f, 390e-9f};
    const float K[3] = {0.686f, 0.678f, 0.666f};
    // TotalRayleigh (CudaSky.h:44-49) and TotalMie (:59-64)
    const float num = 8.f * std::pow(kPi, 3.f) *
                      std::pow(std::pow(sky::kRefractiveIndex, 2.f) - 1.f, 2.f) * (6.f + 3.f * sky::kDepolarization);
    const float c = 0.2f * turbidity * 10e-18f;
    float bR[3], bM[3];
    for (int i = 0; i < 3; ++i) {
        bR[i] = (num / ((3.f * sky::kMolecules) * std::pow(lambda[i], 4.f) * (6.f - 7.f * sky::kDepolarization))) *
                rayleigh;
        bM[i] = (0.434f * c * kPi * std::pow((2.f * kPi) / lambda[i], sky::kMieV - 2.f) * K[i]) * sky::kMieCoefficient;
    }
    v.betaR = make_float3(bR[0], bR[1], bR[2]);
    v.betaM = make_float3(bM[0], bM[1], bM[2]);
    v.betaSum = make_float3(bR[0] + bM[0], bR[1] + bM[1], bR[2] + bM[2]);
    // SunIntensity (CudaSky.h:76-80), Earth shadow falloff at pi / 1.95
    v.sunE = d.sun_intensity *
             std::fmax(0.f, 1.f - std::exp(-(((kPi / 1.95f) - std::acos(cosSunUp)) / sky::kSunFalloffSteepness)));
    const float h = std::pow(1.f - cosSunUp, 5.f);
    v.horizonMix = std::fmin(std::fmax(h, 0.f), 1.f);
    const float t = std::fmax(v.sunDir.y, 0.f);
    sunfade *= (1.f * (1.f - t)) + (0.9f * t);
    v.exponent = 1.f / (1.f + sunfade);
    return v;
}

#ifdef __CUDACC__
// SampleSky (CudaSky.h:105-156) for a unit direction D; black when disabled.
__device__ __forceinline__ float3 sky_radiance(const SkyView& k, const float3& D, bool drawSun)
{
    const float zenith = acosf(fmaxf(D.y, 0.f));  // dot((0, 1, 0), D)
    const float denom = cosf(zenith) + 0.15f * powf(93.885f - ((zenith * 180.f) / kPi), -1.253f);
    const float sR = sky::kRayleighZenithLength / denom;
    const float sM = sky::kMieZenithLength / denom;
    const float3 ex = k.betaR * sR + k.betaM * sM;
    const float3 Fex = make_float3(expf(-ex.x), expf(-ex.y), expf(-ex.z));

    const float cosTheta = dot(D, k.sunDir);
    const float ct = cosTheta * 0.5f + 0.5f;
    const float rayleighPhase = (3.f / (16.f * kPi)) * (1.f + powf(ct, 2.f));
    const float g = sky::kMieG;
    const float hg = (1.f / (4.f * kPi)) *
                     ((1.f - powf(g, 2.f)) / powf(1.f - 2.f * g * cosTheta + powf(g, 2.f), 1.5f));
    const float3 ratio = ((k.betaR * rayleighPhase) + (k.betaM * hg)) / k.betaSum;
    const float3 a = (k.sunE * ratio) * (f3(1.f) - Fex);
    float3 Lin = make_float3(powf(a.x, 1.5f), powf(a.y, 1.5f), powf(a.z, 1.5f));
    const float3 b = (k.sunE * ratio) * Fex;
    const float3 pb = make_float3(powf(b.x, 0.5f), powf(b.y, 0.5f), powf(b.z, 0.5f));
    Lin = Lin * ((f3(1.f) * (1.f - k.horizonMix)) + (pb * k.horizonMix));

    // smoothstep(cos AD, cos AD + 2e-5, cosTheta)
    const float e0 = k.cosSunAngularDiameter, e1 = k.cosSunAngularDiameter + 2e-5f;
    const float y = fmaxf(0.0f, fminf((cosTheta - e0) / (e1 - e0), 1.0f));
    const float sundisk = y * y * (3.0f - (2.0f * y));
    float3 L0 = (f3(0.1f) * Fex) + ((((k.sunE * 19000.f) * Fex) * sundisk) * (drawSun ? 1.f : 0.f));
    // Saturation (CudaSky.h:93-99)
    const float luma = dot(L0, make_float3(0.299f, 0.587f, 0.114f));
    L0 = (f3(luma) * (1.f - 0.5f)) + (L0 * 0.5f);
    // Tonemap (CudaSky.h:85-88)
    const float3 c = Lin + L0;
    const float3 tm = (c * (f3(1.f) + c / f3(1000.f))) / (c + f3(128.f));
    const float3 color = make_float3(fmaxf(0.f, tm.x), fmaxf(0.f, tm.y), fmaxf(0.f, tm.z));
    return make_float3(powf(color.x, k.exponent), powf(color.y, k.exponent), powf(color.z, k.exponent));
}
#endif

}  // namespace tr
