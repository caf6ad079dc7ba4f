// Device closures (BSDF evaluate + sample) of the path-tracing shade kernel.
//
// Restates the reference's closures in tangent space (z = shading normal):
//   Lambert   Tracer/CUDA/GPU/Shade/BSDF/Lambert.h:8-59
//   Diffuse   Tracer/CUDA/GPU/Shade/BSDF/Diffuse.h:8-42
//   Disney    Tracer/CUDA/GPU/Shade/BSDF/Disney.h:30-579 (appleseed Disney BRDF)
//   GGX/GTR1  Tracer/CUDA/GPU/Shade/BSDF/Microfacet.h:33-324
//   finalize  Tracer/CUDA/GPU/Shade/BSDF/Closure.h:57-74
// The arithmetic follows the reference step by step so results agree to
// rounding. REF = true keeps the reference's behaviour where it is
// order-dependent or uses unset values:
//   * Disney::Evaluate writes the diffuse and the sheen value into the same
//     output, so a sheen lobe replaces the diffuse value (Disney.h:416-422);
//   * Disney::Sample feeds the lobe-selection number r0 unchanged to the
//     chosen lobe (Disney.h:491-521) and leaves clearcoat out of the pdf
//     (Disney.h:549-556);
//   * a sample of the sheen, GGX or clearcoat lobe is flagged specular
//     (Disney.h:502,512,520), which skips NEE at this vertex and MIS at the
//     next emissive hit.
// REF = false sums all lobe values, rescales r0 into the chosen lobe's
// interval, includes the clearcoat pdf and flags no Disney lobe as specular
// (none is a delta lobe), so NEE and BSDF sampling always combine by MIS; the
// chosen lobe only picks the direction, which is then evaluated over all lobes
// like the light direction (so a clearcoat sample carries the clearcoat
// Fresnel, where Disney.h:337-366 weights it with the specular one).
// Values the reference leaves unset on early returns are zero in both modes.
#pragma once

#include "tr_device.h"

namespace tr {

struct HitMat {
    float3 diffuse;
    float metallic;
    float3 emissive;
    float subsurface;
    float3 tint;
    float specular;
    float roughness;
    float specularTint;
    float anisotropic;
    float sheen;
    float sheenTint;
    float clearcoat;
    float clearcoatGloss;
    float luminance;
};

struct Lobe {          // BsdfResult
    float3 wi;
    float pdf;
    float3 T;
    uint32_t flags;
};

struct ClosureResult { // Closure
    float3 extT;
    float extPdf;
    float3 extWi;
    uint32_t extFlags;
    float3 shT;
    float shPdf;
};

__device__ __forceinline__ float3 cos_hemisphere(float r0, float r1)
{
    float s, c;
    sincosf(kTwoPi * r0, &s, &c);
    const float b = sqrtf(1.f - r1);
    return make_float3(c * b, s * b, sqrtf(r1));
}

__device__ __forceinline__ ClosureResult finalize_closure(const float3& T, const Lobe& eval, const Lobe& smp)
{
    ClosureResult c;
    c.shT = eval.T * fabsf(eval.wi.z) * T;
    c.shPdf = eval.pdf;
    c.extT = smp.T * fabsf(smp.wi.z) * T;
    c.extPdf = smp.pdf;
    c.extWi = smp.wi;
    c.extFlags = smp.flags;
    return c;
}

// ---------------------------------------------------------------- Lambert
__device__ __forceinline__ ClosureResult lambert_closure(const float3& wo, const float3& wi, const float3& T,
                                                         const HitMat& m, float r0, float r1)
{
    Lobe e;
    const float p = m.roughness < kEpsilon ? 0.f : kRcpPi;
    e.wi = wi;
    e.pdf = p * wi.z;
    e.T = f3(p);
    e.flags = 0;

    Lobe s;
    const float specProb = 1.f - m.roughness;
    if (r0 < specProb) {
        s.wi = make_float3(-wo.x, -wo.y, wo.z);  // reflect(-wo, z)
        s.pdf = 1.f;
        s.T = f3(fdiv(1.f, s.wi.z)) * m.diffuse;
        s.flags = kFlagSpecular;
    } else {
        s.wi = cos_hemisphere(fdiv(specProb - r0, 1.f - specProb), r1);
        s.pdf = kRcpPi * s.wi.z;
        s.T = f3(kRcpPi) * m.diffuse;
        s.flags = 0;
    }
    return finalize_closure(T, e, s);
}

// ---------------------------------------------------------------- Diffuse
__device__ __forceinline__ ClosureResult diffuse_closure(const float3& wo, const float3& wi, const float3& T,
                                                         const HitMat& m, float r0, float r1)
{
    Lobe e;
    e.wi = wi;
    e.pdf = kRcpPi * wi.z;
    e.T = f3(kRcpPi) * m.diffuse;
    e.flags = 0;
    Lobe s;
    s.wi = cos_hemisphere(r0, r1);
    s.pdf = kRcpPi * s.wi.z;
    s.T = f3(kRcpPi) * m.diffuse;
    s.flags = 0;
    return finalize_closure(T, e, s);
}

// ---------------------------------------------------------------- microfacet
namespace mf {

__device__ __forceinline__ void alpha_xy(float roughness, float aniso, float& ax, float& ay)
{
    const float r2 = square(roughness);
    const float aspect = sqrtf(1.0f + aniso * (aniso < 0 ? 0.9f : -0.9f));
    ax = fmaxf(0.001f, fdiv(r2, aspect));
    ay = fmaxf(0.001f, r2 * aspect);
}

__device__ __forceinline__ float stretched_roughness(const float3& m, float sinT, float ax, float ay)
{
    if (ax == ay || sinT == 0.0f)
        return fdiv(1.0f, square(ax));
    return square(fdiv(m.x, sinT * ax)) + square(fdiv(m.z, sinT * ay));
}

__device__ __forceinline__ float projected_roughness(const float3& m, float sinT, float ax, float ay)
{
    if (ax == ay || sinT == 0.0f)
        return ax;
    return sqrtf(square(fdiv(m.x * ax, sinT)) + square(fdiv(m.y * ay, sinT)));
}

__device__ __forceinline__ float ggx_lambda(const float3& v, float ax, float ay)
{
    const float c = v.z;
    if (c == 0.0f)
        return 0.0f;
    const float c2 = square(c);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c2));
    const float a = projected_roughness(v, s, ax, ay);
    const float t2 = fdiv(square(s), c2);
    return (-1.0f + sqrtf(1.0f + square(a) * t2)) * 0.5f;
}

__device__ __forceinline__ float ggx_D(const float3& m, float ax, float ay)
{
    const float c = m.z;
    if (c == 0.0f)
        return square(ax) * kRcpPi;
    const float c2 = square(c);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c2));
    const float c4 = square(c2);
    const float t2 = fdiv(1.0f - c2, c2);
    const float A = stretched_roughness(m, s, ax, ay);
    const float tmp = 1.0f + t2 * A;
    return fdiv(1.0f, kPi * ax * ay * c4 * square(tmp));
}

__device__ __forceinline__ float ggx_G(const float3& wi, const float3& wo, float ax, float ay)
{
    return fdiv(1.0f, 1.0f + ggx_lambda(wo, ax, ay) + ggx_lambda(wi, ax, ay));
}

__device__ __forceinline__ float ggx_pdf(const float3& v, const float3& m, float ax, float ay)
{
    if (v.z == 0.0f)
        return 0.0f;
    const float G1 = fdiv(1.0f, 1.0f + ggx_lambda(v, ax, ay));
    return fdiv(G1 * fabsf(dot(v, m)) * ggx_D(m, ax, ay), fabsf(v.z));
}

// visible-normal sample (Heitz 2017), Microfacet.h:172-210
__device__ __forceinline__ float3 ggx_sample(const float3& v, float r0, float r1, float ax, float ay)
{
    const float sgn = v.z < 0.0f ? -1.0f : 1.0f;
    const float3 st = normalize(make_float3(sgn * v.x * ax, sgn * v.y * ay, sgn * v.z));
    const float3 t1 = v.y < 0.9999f ? normalize(cross(st, make_float3(0.f, 0.f, 1.f))) : make_float3(1.f, 0.f, 0.f);
    const float3 t2 = cross(t1, st);
    const float a = fdiv(1.0f, 1.0f + st.z);
    const float r = sqrtf(r0);
    const float phi = r1 < a ? fdiv(r1, a) * kPi : kPi + fdiv(r1 - a, 1.0f - a) * kPi;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const float p1 = r * cp;
    const float p2 = r * sp * (r1 < a ? 1.0f : st.z);
    const float3 h = p1 * t1 + p2 * t2 + sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2)) * st;
    return normalize(make_float3(h.x * ax, h.y * ay, fmaxf(0.0f, h.z)));
}

__device__ __forceinline__ float gtr1_lambda(const float3& v, float ax)
{
    const float c = v.z;
    if (c == 0.0f)
        return 0.0f;
    const float c2 = square(c);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c2));
    if (s == 0.0f)
        return 0.0f;
    const float cot2 = fdiv(c2, square(s));
    const float cot = sqrtf(cot2);
    const float alpha = clampf(ax, 0.001f, 0.999f);
    const float a2 = square(alpha);
    const float a = sqrtf(cot2 + a2);
    const float b = sqrtf(cot2 + 1.0f);
    const float lc = logf(cot + b);
    const float ld = logf(cot + a);
    return fdiv(a - b + cot * (lc - ld), cot * logf(a2));
}

__device__ __forceinline__ float gtr1_D(const float3& m, float ax)
{
    const float alpha = clampf(ax, 0.001f, 0.999f);
    const float a2 = square(alpha);
    const float c2 = square(m.z);
    const float a = fdiv(a2 - 1.0f, kPi * logf(a2));
    const float b = fdiv(1.0f, 1.0f + (a2 - 1.0f) * c2);
    return a * b;
}

__device__ __forceinline__ float gtr1_G(const float3& wi, const float3& wo, float ax)
{
    return fdiv(1.0f, 1.0f + gtr1_lambda(wo, ax) + gtr1_lambda(wi, ax));
}

// GTR1 pdf as stated in the reference (Microfacet.h:320-323; uses |m.y|)
__device__ __forceinline__ float gtr1_pdf(const float3& m, float ax) { return gtr1_D(m, ax) * fabsf(m.y); }

__device__ __forceinline__ float3 gtr1_sample(float r0, float r1, float ax)
{
    const float alpha = clampf(ax, 0.001f, 0.999f);
    const float a2 = square(alpha);
    const float a = 1.0f - powf(a2, 1.0f - r0);
    const float c2 = fdiv(a, 1.0f - a2);
    const float c = sqrtf(c2);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c2));
    float sp, cp;
    sincosf(kTwoPi * r1, &sp, &cp);
    return make_float3(cp * s, sp * s, c);
}

} // namespace mf

// ---------------------------------------------------------------- Disney
namespace disney {

__device__ __forceinline__ float schlick(float u)
{
    const float m = saturate(1.0f - u);
    const float m2 = square(m);
    return square(m2) * m;
}

__device__ __forceinline__ float3 spec_fresnel(const HitMat& mat, const float3& o, const float3& h)
{
    float3 v = (1.f - mat.specularTint) + mat.specularTint * mat.tint;
    v *= mat.specular * 0.08f;
    v = ((1.f - mat.metallic) * v) + (mat.metallic * mat.diffuse);
    const float f = schlick(fabsf(dot(o, h)));
    return ((1.f - f) * v) + f;
}

__device__ __forceinline__ float3 clearcoat_fresnel(const HitMat& mat, const float3& o, const float3& h)
{
    const float f = schlick(fabsf(dot(o, h)));
    return f3(mix(0.04f, 1.0f, f) * 0.25f * mat.clearcoat);
}

__device__ __forceinline__ bool force_above(float3& d)
{
    const float corr = 1.0e-4f - d.z;
    if (corr <= 0)
        return false;
    d = normalize(d + corr * make_float3(0.f, 0.f, 1.f));
    return true;
}

__device__ __forceinline__ float diffuse_eval(const HitMat& mat, const float3& wo, const float3& wi, float3& value)
{
    const float3 h = normalize(wi + wo);
    const float con = wo.z, cin = wi.z, cih = dot(wi, h);
    const float fl = schlick(cin), fv = schlick(con);
    float fd = 0.0f;
    if (mat.subsurface != 1.0f) {
        const float fd90 = 0.5f + 2.0f * square(cih) * mat.roughness;
        fd = mix(1.0f, fd90, fl) * mix(1.0f, fd90, fv);
    }
    if (mat.subsurface > 0.0f) {
        const float fss90 = square(cih) * mat.roughness;
        const float fss = mix(1.0f, fss90, fl) * mix(1.0f, fss90, fv);
        const float ss = 1.25f * (fss * (fdiv(1.0f, fabsf(con) + fabsf(cin)) - 0.5f) + 0.5f);
        fd = mix(fd, ss, mat.subsurface);
    }
    value = mat.diffuse;
    value *= fd * kRcpPi * (1.0f - mat.metallic);
    return fabsf(cin) * kRcpPi;
}

__device__ __forceinline__ float sheen_eval(const HitMat& mat, const float3& wo, const float3& wi, float3& value)
{
    const float3 h = normalize(wi + wo);
    const float fh = schlick(dot(wi, h));
    value = (1.f - mat.sheenTint) + mat.sheenTint * mat.tint;
    value *= fh * mat.sheen * (1.0f - mat.metallic);
    return kRcpTwoPi;
}

__device__ __forceinline__ float ggx_eval(float ax, float ay, const HitMat& mat, const float3& wo, const float3& wi,
                                          float3& value)
{
    if (wo.z == 0.0f || wi.z == 0.0f)
        return 0.0f;
    const float3 m = normalize(wi + wo);
    const float coh = dot(wo, m);
    if (coh == 0.0f)
        return 0.0f;
    const float D = mf::ggx_D(m, ax, ay);
    const float G = mf::ggx_G(wi, wo, ax, ay);
    value = spec_fresnel(mat, wo, m);
    value *= fdiv(D * G, fabsf(4.0f * wo.z * wi.z));
    return fdiv(mf::ggx_pdf(wo, m, ax, ay), fabsf(4.0f * coh));
}

__device__ __forceinline__ void ggx_sample(float ax, float ay, const HitMat& mat, float r0, float r1, const float3& wo,
                                           float3& wi, float& pdf, float3& value)
{
    if (wo.z == 0.0f)
        return;
    float3 m = mf::ggx_sample(wo, r0, r1, ax, ay);
    wi = reflect(-wo, m);
    if (force_above(wi))
        m = normalize(wo + wi);
    if (wi.z == 0.0f)
        return;
    const float coh = dot(wo, m);
    pdf = fdiv(mf::ggx_pdf(wo, m, ax, ay), fabsf(4.0f * coh));
    if (pdf < 1e-6f)
        return;
    const float D = mf::ggx_D(m, ax, ay);
    const float G = mf::ggx_G(wi, wo, ax, ay);
    value = spec_fresnel(mat, wo, m);
    value *= fdiv(D * G, fabsf(4.0f * wo.z * wi.z));
}

__device__ __forceinline__ float gtr1_eval(float a, const HitMat& mat, const float3& wo, const float3& wi, float3& value)
{
    if (wo.z == 0.0f || wi.z == 0.0f)
        return 0.0f;
    const float3 m = normalize(wi + wo);
    const float coh = dot(wo, m);
    if (coh == 0.0f)
        return 0.0f;
    const float D = mf::gtr1_D(m, a);
    const float G = mf::gtr1_G(wi, wo, a);
    value = clearcoat_fresnel(mat, wo, m);
    value *= fdiv(D * G, fabsf(4.0f * wo.z * wi.z));
    return fdiv(mf::gtr1_pdf(m, a), fabsf(4.0f * coh));
}

// Disney.h:337-366: the clearcoat sample is weighted with the specular Fresnel
__device__ __forceinline__ void gtr1_sample(float a, const HitMat& mat, float r0, float r1, const float3& wo, float3& wi,
                                            float& pdf, float3& value)
{
    if (wo.z == 0.0f)
        return;
    float3 m = mf::gtr1_sample(r0, r1, a);
    wi = reflect(-wo, m);
    if (force_above(wi))
        m = normalize(wo + wi);
    if (wi.z == 0.0f)
        return;
    const float coh = dot(wo, m);
    pdf = fdiv(mf::gtr1_pdf(m, a), fabsf(4.0f * coh));
    if (pdf < 1e-6f)
        return;
    const float D = mf::gtr1_D(m, a);
    const float G = mf::gtr1_G(wi, wo, a);
    value = spec_fresnel(mat, wo, m);
    value *= fdiv(D * G, fabsf(4.0f * wo.z * wi.z));
}

__device__ __forceinline__ bool weights(const HitMat& mat, float& wd, float& ws, float& wsp, float& wc)
{
    wd = lerp(mat.luminance, 0.f, mat.metallic);
    ws = lerp(mat.sheen, 0.f, mat.metallic);
    wsp = lerp(mat.specular, 1.f, mat.metallic);
    wc = mat.clearcoat * .25f;
    const float total = wd + ws + wsp + wc;
    if (total == 0.0f)
        return false;
    const float rcp = fdiv(1.f, total);
    wd *= rcp;
    ws *= rcp;
    wsp *= rcp;
    wc *= rcp;
    return true;
}

__device__ __forceinline__ float clearcoat_alpha(const HitMat& mat) { return mix(0.1f, 0.001f, mat.clearcoatGloss); }

template <bool REF>
__device__ __forceinline__ Lobe evaluate(const float3& wo, const float3& wi, const HitMat& mat)
{
    Lobe r;
    r.wi = wi;
    r.pdf = 0.f;
    r.T = f3(0.f);
    r.flags = 0;
    float wd, ws, wsp, wc;
    if (!weights(mat, wd, ws, wsp, wc))
        return r;
    float pdf = 0.f;
    float3 incoming = f3(0.f);
    if (REF) {
        // the diffuse and sheen evaluations share one output value
        if (wd > 0)
            pdf += wd * diffuse_eval(mat, wo, wi, incoming);
        if (ws > 0)
            pdf += ws * sheen_eval(mat, wo, wi, incoming);
    } else {
        float3 v = f3(0.f);
        if (wd > 0) {
            pdf += wd * diffuse_eval(mat, wo, wi, v);
            incoming += v;
        }
        if (ws > 0) {
            pdf += ws * sheen_eval(mat, wo, wi, v);
            incoming += v;
        }
    }
    if (wsp > 0) {
        float ax, ay;
        mf::alpha_xy(mat.roughness, mat.anisotropic, ax, ay);
        float3 v = f3(0.f);
        const float p = ggx_eval(ax, ay, mat, wo, wi, v);
        if (p > 0) {
            pdf += wsp * p;
            incoming += v;
        }
    }
    if (wc > 0) {
        float3 v = f3(0.f);
        const float p = gtr1_eval(clearcoat_alpha(mat), mat, wo, wi, v);
        if (p > 0) {
            pdf += wc * p;
            incoming += v;
        }
    }
    r.pdf = pdf;
    r.T = incoming;
    return r;
}

template <bool REF>
__device__ __forceinline__ Lobe sample(const float3& wo, const HitMat& mat, float r0, float r1)
{
    Lobe r;
    r.wi = make_float3(0.f, 0.f, 1.f);
    r.pdf = 0.f;
    r.T = f3(0.f);
    r.flags = 0;
    float wd, ws, wsp, wc;
    if (!weights(mat, wd, ws, wsp, wc))
        return r;
    const float cd = wd, cs = cd + ws, csp = cs + wsp;

    float3 wi = make_float3(0.f, 0.f, 1.f);
    float prob = 0.f, cpdf = 0.f;
    float3 value = f3(0.f);
    uint32_t flags = 0;
    if (r0 < cd) {
        const float u = REF ? r0 : fdiv(r0, wd);
        wi = cos_hemisphere(u, r1);
        cpdf = diffuse_eval(mat, wo, wi, value);
        prob = wd * cpdf;
        wd = 0;
    } else if (r0 < cs) {
        const float u = REF ? r0 : fdiv(r0 - cd, ws);
        wi = cos_hemisphere(u, r1);
        cpdf = sheen_eval(mat, wo, wi, value);
        prob = ws * cpdf;
        ws = 0;
        flags |= REF ? kFlagSpecular : 0u;
    } else if (r0 < csp) {
        const float u = REF ? r0 : fminf_(fdiv(r0 - cs, wsp), 0.99999994f);
        float ax, ay;
        mf::alpha_xy(mat.roughness, mat.anisotropic, ax, ay);
        ggx_sample(ax, ay, mat, u, r1, wo, wi, cpdf, value);
        prob = wsp * cpdf;
        wsp = 0;
        flags |= REF ? kFlagSpecular : 0u;
    } else {
        const float u = REF ? r0 : fminf_(fdiv(r0 - csp, wc), 0.99999994f);
        gtr1_sample(clearcoat_alpha(mat), mat, u, r1, wo, wi, cpdf, value);
        prob = wc * cpdf;
        wc = 0;
        flags |= REF ? kFlagSpecular : 0u;
    }
    if (wd > 0) {
        float3 v;
        prob += wd * diffuse_eval(mat, wo, wi, v);
        value += v;
    }
    if (ws > 0) {
        float3 v;
        prob += ws * sheen_eval(mat, wo, wi, v);
        value += v;
    }
    if (wsp > 0) {
        float ax, ay;
        mf::alpha_xy(mat.roughness, mat.anisotropic, ax, ay);
        float3 v = f3(0.f);
        prob += wsp * ggx_eval(ax, ay, mat, wo, wi, v);
        value += v;
    }
    if (wc > 0) {
        float3 v = f3(0.f);
        const float p = gtr1_eval(clearcoat_alpha(mat), mat, wo, wi, v);
        if (!REF)
            prob += wc * p;
        value += v;
    }
    r.wi = wi;
    r.pdf = prob > 1e-6f ? prob : 0;
    r.T = value;
    r.flags = flags;
    return r;
}

} // namespace disney

// ---------------------------------------------------------------- Disney, default sampling mode
// The default mode's closure: the sampled lobe only chooses the direction, and
// the light direction and the sampled direction are both evaluated over all
// lobes (value = sum of the lobe values, pdf = sum of weight x lobe pdf), so
// the extend direction's value is the closure value that the path-replay
// adjoint differentiates. The terms that depend on the material and wo alone
// (lobe weights, alphas, the Smith Lambda of wo, the GTR1 normalisation) are
// computed once per hit; each term is the same arithmetic as in
// disney::evaluate<false>.
namespace disney {

struct Prep {
    float wd, ws, wsp, wc;  // lobe selection weights
    float ax, ay;           // GGX alphas (Microfacet.h:33-49)
    float lamO;             // GGX Lambda(wo)
    float ccA;              // GTR1 alpha before its clamp
    float ccA2;             // clamped GTR1 alpha squared
    float ccLogA2;          // log(ccA2)
    float ccNorm;           // (a2 - 1) / (pi log a2) of GTR1's D
    float ccLamO;           // GTR1 Lambda(wo)
};

__device__ __forceinline__ float gtr1_lambda_c(const float3& v, float a2, float logA2)
{
    const float c = v.z;
    if (c == 0.0f)
        return 0.0f;
    const float c2 = square(c);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - c2));
    if (s == 0.0f)
        return 0.0f;
    const float cot2 = fdiv(c2, square(s));
    const float cot = sqrtf(cot2);
    const float a = sqrtf(cot2 + a2);
    const float b = sqrtf(cot2 + 1.0f);
    const float lc = logf(cot + b);
    const float ld = logf(cot + a);
    return fdiv(a - b + cot * (lc - ld), cot * logA2);
}

__device__ __forceinline__ bool prepare(const HitMat& mat, const float3& wo, Prep& p)
{
    if (!weights(mat, p.wd, p.ws, p.wsp, p.wc))
        return false;
    mf::alpha_xy(mat.roughness, mat.anisotropic, p.ax, p.ay);
    p.lamO = p.wsp > 0 ? mf::ggx_lambda(wo, p.ax, p.ay) : 0.f;
    p.ccA = clearcoat_alpha(mat);
    if (p.wc > 0) {
        const float alpha = clampf(p.ccA, 0.001f, 0.999f);
        p.ccA2 = square(alpha);
        p.ccLogA2 = logf(p.ccA2);
        p.ccNorm = fdiv(p.ccA2 - 1.0f, kPi * p.ccLogA2);
        p.ccLamO = gtr1_lambda_c(wo, p.ccA2, p.ccLogA2);
    }
    return true;
}

// ggx_eval with Lambda(wo) and D computed once
__device__ __forceinline__ float ggx_eval_p(const Prep& p, const HitMat& mat, const float3& wo, const float3& wi,
                                            float3& value)
{
    if (wo.z == 0.0f || wi.z == 0.0f)
        return 0.0f;
    const float3 m = normalize(wi + wo);
    const float coh = dot(wo, m);
    if (coh == 0.0f)
        return 0.0f;
    const float D = mf::ggx_D(m, p.ax, p.ay);
    const float G = fdiv(1.0f, 1.0f + p.lamO + mf::ggx_lambda(wi, p.ax, p.ay));
    value = spec_fresnel(mat, wo, m);
    value *= fdiv(D * G, fabsf(4.0f * wo.z * wi.z));
    const float G1 = fdiv(1.0f, 1.0f + p.lamO);
    return fdiv(fdiv(G1 * fabsf(coh) * D, fabsf(wo.z)), fabsf(4.0f * coh));
}

// gtr1_eval with the GTR1 normalisation, Lambda(wo) and D computed once
__device__ __forceinline__ float gtr1_eval_p(const Prep& p, const HitMat& mat, const float3& wo, const float3& wi,
                                             float3& value)
{
    if (wo.z == 0.0f || wi.z == 0.0f)
        return 0.0f;
    const float3 m = normalize(wi + wo);
    const float coh = dot(wo, m);
    if (coh == 0.0f)
        return 0.0f;
    const float D = p.ccNorm * fdiv(1.0f, 1.0f + (p.ccA2 - 1.0f) * square(m.z));
    const float G = fdiv(1.0f, 1.0f + p.ccLamO + gtr1_lambda_c(wi, p.ccA2, p.ccLogA2));
    value = clearcoat_fresnel(mat, wo, m);
    value *= fdiv(D * G, fabsf(4.0f * wo.z * wi.z));
    return fdiv(D * fabsf(m.y), fabsf(4.0f * coh));
}

// All lobes at wi: returns sum(weight x pdf), value = sum of the lobe values (evaluate<false>).
__device__ __forceinline__ float eval_all(const Prep& p, const HitMat& mat, const float3& wo, const float3& wi,
                                          float3& value)
{
    float pdf = 0.f;
    value = f3(0.f);
    float3 v = f3(0.f);
    if (p.wd > 0) {
        pdf += p.wd * diffuse_eval(mat, wo, wi, v);
        value += v;
    }
    if (p.ws > 0) {
        pdf += p.ws * sheen_eval(mat, wo, wi, v);
        value += v;
    }
    if (p.wsp > 0) {
        v = f3(0.f);
        const float q = ggx_eval_p(p, mat, wo, wi, v);
        if (q > 0) {
            pdf += p.wsp * q;
            value += v;
        }
    }
    if (p.wc > 0) {
        v = f3(0.f);
        const float q = gtr1_eval_p(p, mat, wo, wi, v);
        if (q > 0) {
            pdf += p.wc * q;
            value += v;
        }
    }
    return pdf;
}

// The sampled direction: the lobe r0 falls in, with r0 rescaled into its interval.
__device__ __forceinline__ float3 sample_direction(const Prep& p, const float3& wo, float r0, float r1)
{
    const float cd = p.wd, cs = cd + p.ws, csp = cs + p.wsp;
    float3 wi = make_float3(0.f, 0.f, 1.f);
    if (r0 < cd) {
        wi = cos_hemisphere(fdiv(r0, p.wd), r1);
    } else if (r0 < cs) {
        wi = cos_hemisphere(fdiv(r0 - cd, p.ws), r1);
    } else if (wo.z != 0.0f) {
        float3 m;
        if (r0 < csp)
            m = mf::ggx_sample(wo, fminf_(fdiv(r0 - cs, p.wsp), 0.99999994f), r1, p.ax, p.ay);
        else
            m = mf::gtr1_sample(fminf_(fdiv(r0 - csp, p.wc), 0.99999994f), r1, p.ccA);
        wi = reflect(-wo, m);
        force_above(wi);
    }
    return wi;
}

} // namespace disney

// evalLight = false (default mode): the light direction is not evaluated (its
// result would be discarded: the light sample has no density there).
template <bool REF>
__device__ __forceinline__ ClosureResult disney_closure(const float3& wo, const float3& wi, const float3& T,
                                                        const HitMat& m, float r0, float r1, bool evalLight = true)
{
    if (REF) {
        const Lobe e = disney::evaluate<REF>(wo, wi, m);
        const Lobe s = disney::sample<REF>(wo, m, r0, r1);
        return finalize_closure(T, e, s);
    }
    Lobe e, s;
    e.wi = wi;
    e.pdf = 0.f;
    e.T = f3(0.f);
    e.flags = 0;
    s.wi = make_float3(0.f, 0.f, 1.f);
    s.pdf = 0.f;
    s.T = f3(0.f);
    s.flags = 0;
    disney::Prep p;
    if (disney::prepare(m, wo, p)) {
        if (evalLight)
            e.pdf = disney::eval_all(p, m, wo, wi, e.T);
        s.wi = disney::sample_direction(p, wo, r0, r1);
        const float q = disney::eval_all(p, m, wo, s.wi, s.T);
        s.pdf = q > 1e-6f ? q : 0.f;
    }
    return finalize_closure(T, e, s);
}

} // namespace tr
