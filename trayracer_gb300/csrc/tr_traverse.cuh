// Closest-hit and any-hit traversal of the 8-wide BVH (the compressed wide BVH's
// child and leaf encoding, child boxes in fp32 or 8-bit quantized).
//
// Replaces optixTrace (Tracer/Optix/GPU/optix.cu:264,308,333) with a software
// traversal following Ylitie, Karras and Laine (HPG 2017): node groups on a
// short stack, octant-ordered child slots, 8-bit quantized child boxes decoded
// against the ray with one FMA per slab, leaf triangles visited as a bit mask.
// Node words are fetched as 128-bit read-only loads.
//
// OptiX semantics kept: no face culling (Tracer/Resources/Model.cpp:270),
// closest hit over [tmin, tmax], any-hit termination for shadow rays
// (OPTIX_RAY_FLAG_TERMINATE_ON_FIRST_HIT, optix.cu:333-335).
//
// The triangle test is Moller-Trumbore on (v0, e1 = v1 - v0, e2 = v2 - v0)
// written with explicit round-to-nearest operations (no contraction choice
// left to the compiler), so the oracle's host copy of the same sequence gives
// bit-identical t, u, v.
#pragma once

#include <cmath>

#include "tr_device.h"

namespace tr {

// Round-to-nearest arithmetic and bit operations with one meaning on the
// device and on the host (the host copy is built with -ffp-contract=off).
TR_HD float fma_rn(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
TR_HD float mul_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
TR_HD float add_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
TR_HD float sub_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
TR_HD float rcp_rn(float a)
{
#if defined(__CUDA_ARCH__)
    return __frcp_rn(a);
#else
    return 1.0f / a;
#endif
}
TR_HD uint32_t clz32(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return uint32_t(__clz(x));
#else
    return x ? uint32_t(__builtin_clz(x)) : 32u;
#endif
}
TR_HD uint32_t popc32(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return uint32_t(__popc(x));
#else
    return uint32_t(__builtin_popcount(x));
#endif
}
TR_HD uint32_t ffs32(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return uint32_t(__ffs(x));
#else
    return uint32_t(__builtin_ffs(int(x)));
#endif
}
template <class T> TR_HD T ldg(const T* p)
{
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}

// Traversal work of one ray (counting variant only).
struct TraversalCounts {
    uint32_t nodes;
    uint32_t tris;
};

constexpr int kTraversalStack = 32;

struct TriHit {
    float t;
    float u;
    float v;
    uint32_t slot;
};

TR_HD bool intersect_triangle(const float3& O, const float3& D, const float4& a, const float4& b,
                                                   const float4& c, float tmin, float tmax, float& t, float& u, float& v)
{
    // pvec = D x e2
    const float px = fma_rn(D.y, c.z, -mul_rn(D.z, c.y));
    const float py = fma_rn(D.z, c.x, -mul_rn(D.x, c.z));
    const float pz = fma_rn(D.x, c.y, -mul_rn(D.y, c.x));
    const float det = fma_rn(b.x, px, fma_rn(b.y, py, mul_rn(b.z, pz)));
    if (det == 0.0f)
        return false;
    const float inv = rcp_rn(det);
    const float tx = sub_rn(O.x, a.x);
    const float ty = sub_rn(O.y, a.y);
    const float tz = sub_rn(O.z, a.z);
    const float uu = mul_rn(fma_rn(tx, px, fma_rn(ty, py, mul_rn(tz, pz))), inv);
    if (!(uu >= 0.0f && uu <= 1.0f))
        return false;
    // qvec = tvec x e1
    const float qx = fma_rn(ty, b.z, -mul_rn(tz, b.y));
    const float qy = fma_rn(tz, b.x, -mul_rn(tx, b.z));
    const float qz = fma_rn(tx, b.y, -mul_rn(ty, b.x));
    const float vv = mul_rn(fma_rn(D.x, qx, fma_rn(D.y, qy, mul_rn(D.z, qz))), inv);
    if (!(vv >= 0.0f && add_rn(uu, vv) <= 1.0f))
        return false;
    const float tt = mul_rn(fma_rn(c.x, qx, fma_rn(c.y, qy, mul_rn(c.z, qz))), inv);
    if (!(tt >= tmin && tt <= tmax))
        return false;
    t = tt;
    u = uu;
    v = vv;
    return true;
}

// float(byte i of w), exact. On the device the byte is placed in the low
// mantissa bits of 2^23 (one byte permute) and 2^23 subtracted (one add), which
// avoids the quarter-rate integer-to-float conversion.
TR_HD float byte_to_float(uint32_t w, int i)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(__byte_perm(w, 0x4B00u, 0x5440u | uint32_t(i))) - 8388608.0f;
#else
    return float((w >> (8 * i)) & 0xffu);
#endif
}

#ifdef __CUDA_ARCH__
// Packed fp32 pairs (sm_100 and later): lane 0 in the low word.
__device__ __forceinline__ unsigned long long pack2(float lo, float hi)
{
    unsigned long long d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ void unpack2(unsigned long long v, float& lo, float& hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b)
{
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// Byte j of lo and of hi, each placed in the low mantissa bits of 2^23.
__device__ __forceinline__ unsigned long long byte_pair(uint32_t lo, uint32_t hi, int j)
{
    const uint32_t a = __byte_perm(lo, 0x4B00u, 0x5440u | uint32_t(j));
    const uint32_t b = __byte_perm(hi, 0x4B00u, 0x5440u | uint32_t(j));
    unsigned long long d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "r"(a), "r"(b));
    return d;
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b)
{
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b)
{
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ float max3(float a, float b, float c)
{
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
#endif

// Intersects the 8 children of a node; returns the hit mask: bits 24..31 for
// internal children (position 24 + (slot ^ (7 - octant))), bits 0..23 for
// leaf triangles (offset from the node's triangle base). imask gets the
// node's internal children (bit per slot). A child plane's distance is
// (plane - O) * invD with each operation rounded (the slab test of Ize,
// "Robust BVH Ray Traversal", JCGT 2013: the far distance is scaled by
// 1 + 2^-21.3 before the comparison to cover the rounding of both distances).
TR_HD uint32_t intersect_wnode(const WideNode* __restrict__ nodes, uint32_t nodeIx,
                                                   const float3& O, const float3& invD, uint32_t octInv, float tmin,
                                                   float tmax, uint32_t& childBase, uint32_t& triBase,
                                                   uint32_t& imask)
{
    const WideNode* node = nodes + nodeIx;
    const uint4 h = ldg(&node->hdr);
    childBase = h.x;
    triBase = h.y;
    // the near plane is hi on axes the ray walks backwards
    const bool nx = invD.x < 0.f, ny = invD.y < 0.f, nz = invD.z < 0.f;
    const float* nearX = nx ? node->hi[0] : node->lo[0];
    const float* farX = nx ? node->lo[0] : node->hi[0];
    const float* nearY = ny ? node->hi[1] : node->lo[1];
    const float* farY = ny ? node->lo[1] : node->hi[1];
    const float* nearZ = nz ? node->hi[2] : node->lo[2];
    const float* farZ = nz ? node->lo[2] : node->hi[2];
#ifdef __CUDA_ARCH__
    const unsigned long long ox2 = pack2(O.x, O.x), oy2 = pack2(O.y, O.y), oz2 = pack2(O.z, O.z);
    const unsigned long long ix2 = pack2(invD.x, invD.x), iy2 = pack2(invD.y, invD.y), iz2 = pack2(invD.z, invD.z);
#endif

    // Per byte of meta: the hit-mask bit position (internal children, whose
    // low five bits are >= 24, are re-ordered by the ray octant) and the bits
    // to set there (the unary triangle count, or one bit for an internal
    // child; zero for an empty slot, so empty slots need no branch).
    const uint32_t octInv4 = octInv * 0x01010101u;
    uint32_t hitmask = 0;
    imask = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const uint32_t meta4 = half == 0 ? h.z : h.w;
        const uint32_t inner4 = ((meta4 & (meta4 << 1)) & 0x10101010u) >> 4;  // 1 per internal child
        // the four 0/1 bytes gathered into bits 28..31 by one multiply
        imask |= ((inner4 * 0x10204080u) >> 28) << (4 * half);
        const uint32_t bitIndex4 = (meta4 ^ (octInv4 & (inner4 * 0xffu))) & 0x1f1f1f1fu;
        const uint32_t childBits4 = (meta4 >> 5) & 0x07070707u;
        float t0x[4], t1x[4], t0y[4], t1y[4], t0z[4], t1z[4];
#ifdef __CUDA_ARCH__
        const float4 nX = ldg(reinterpret_cast<const float4*>(nearX) + half);
        const float4 fX = ldg(reinterpret_cast<const float4*>(farX) + half);
        const float4 nY = ldg(reinterpret_cast<const float4*>(nearY) + half);
        const float4 fY = ldg(reinterpret_cast<const float4*>(farY) + half);
        const float4 nZ = ldg(reinterpret_cast<const float4*>(nearZ) + half);
        const float4 fZ = ldg(reinterpret_cast<const float4*>(farZ) + half);
        // two children per packed subtract and multiply (each lane rounds as the
        // scalar sub_rn / mul_rn do)
        auto slab = [&](const float4& p, unsigned long long o2, unsigned long long i2, float (&t)[4]) {
            unpack2(mul2(sub2(pack2(p.x, p.y), o2), i2), t[0], t[1]);
            unpack2(mul2(sub2(pack2(p.z, p.w), o2), i2), t[2], t[3]);
        };
        slab(nX, ox2, ix2, t0x);
        slab(fX, ox2, ix2, t1x);
        slab(nY, oy2, iy2, t0y);
        slab(fY, oy2, iy2, t1y);
        slab(nZ, oz2, iz2, t0z);
        slab(fZ, oz2, iz2, t1z);
#else
        for (int j = 0; j < 4; ++j) {
            const int sl = 4 * half + j;
            t0x[j] = mul_rn(sub_rn(nearX[sl], O.x), invD.x);
            t1x[j] = mul_rn(sub_rn(farX[sl], O.x), invD.x);
            t0y[j] = mul_rn(sub_rn(nearY[sl], O.y), invD.y);
            t1y[j] = mul_rn(sub_rn(farY[sl], O.y), invD.y);
            t0z[j] = mul_rn(sub_rn(nearZ[sl], O.z), invD.z);
            t1z[j] = mul_rn(sub_rn(farZ[sl], O.z), invD.z);
        }
#endif
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#ifdef __CUDA_ARCH__
            const float tn = max3(t0x[j], t0y[j], fmaxf(t0z[j], tmin));
            const float tf = min3(t1x[j], t1y[j], fminf(t1z[j], tmax));
#else
            const float tn = fmaxf(fmaxf(t0x[j], t0y[j]), fmaxf(t0z[j], tmin));
            const float tf = fminf(fminf(t1x[j], t1y[j]), fminf(t1z[j], tmax));
#endif
            if (tn <= tf * 1.0000004f)
                hitmask |= ((childBits4 >> (8 * j)) & 7u) << ((bitIndex4 >> (8 * j)) & 31u);
        }
    }
    return hitmask;
}

// The same for a node with 8-bit quantized child boxes (the compressed wide BVH
// of Ylitie et al.): a child plane is p + q * 2^e of the node's origin and
// exponents, its distance one fused multiply-add of the byte.
TR_HD uint32_t intersect_qnode(const QuantNode* __restrict__ nodes, uint32_t nodeIx,
                                                   const float3& O, const float3& invD, uint32_t octInv, float tmin,
                                                   float tmax, uint32_t& childBase, uint32_t& triBase,
                                                   uint32_t& imask)
{
    const uint4* nw = reinterpret_cast<const uint4*>(nodes + nodeIx);
    const uint4 w0 = ldg(nw + 0);
    const uint4 w1 = ldg(nw + 1);
    const uint4 w2 = ldg(nw + 2);
    const uint4 w3 = ldg(nw + 3);
    const uint4 w4 = ldg(nw + 4);

    const float px = u2f(w0.x), py = u2f(w0.y), pz = u2f(w0.z);
    const float sx = u2f((w0.w & 0xffu) << 23);
    const float sy = u2f(((w0.w >> 8) & 0xffu) << 23);
    const float sz = u2f(((w0.w >> 16) & 0xffu) << 23);
    imask = w0.w >> 24;
    childBase = w1.x;
    triBase = w1.y;

    const float ax = sx * invD.x, ay = sy * invD.y, az = sz * invD.z;
    const float bx = (px - O.x) * invD.x, by = (py - O.y) * invD.y, bz = (pz - O.z) * invD.z;
#ifdef __CUDA_ARCH__
    const unsigned long long ax2 = pack2(ax, ax), ay2 = pack2(ay, ay), az2 = pack2(az, az);
    const unsigned long long bx2 = pack2(bx, bx), by2 = pack2(by, by), bz2 = pack2(bz, bz);
    const unsigned long long kMinus2p23x2 = pack2(-8388608.0f, -8388608.0f);
#endif

    // octant swizzle: the near plane is qhi on axes the ray walks backwards
    const bool nx = invD.x < 0.f, ny = invD.y < 0.f, nz = invD.z < 0.f;
    const uint32_t loX0 = nx ? w3.z : w2.x, loX1 = nx ? w3.w : w2.y;
    const uint32_t hiX0 = nx ? w2.x : w3.z, hiX1 = nx ? w2.y : w3.w;
    const uint32_t loY0 = ny ? w4.x : w2.z, loY1 = ny ? w4.y : w2.w;
    const uint32_t hiY0 = ny ? w2.z : w4.x, hiY1 = ny ? w2.w : w4.y;
    const uint32_t loZ0 = nz ? w4.z : w3.x, loZ1 = nz ? w4.w : w3.y;
    const uint32_t hiZ0 = nz ? w3.x : w4.z, hiZ1 = nz ? w3.y : w4.w;

    // Per byte of meta: the hit-mask bit position (internal children, whose
    // low five bits are >= 24, are re-ordered by the ray octant) and the bits
    // to set there (the unary triangle count, or one bit for an internal
    // child; zero for an empty slot, so empty slots need no branch).
    const uint32_t octInv4 = octInv * 0x01010101u;
    uint32_t hitmask = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const uint32_t meta4 = half == 0 ? w1.z : w1.w;
        const uint32_t inner4 = ((meta4 & (meta4 << 1)) & 0x10101010u) >> 4;  // 1 per internal child
        const uint32_t bitIndex4 = (meta4 ^ (octInv4 & (inner4 * 0xffu))) & 0x1f1f1f1fu;
        const uint32_t childBits4 = (meta4 >> 5) & 0x07070707u;
        const uint32_t lx = half == 0 ? loX0 : loX1, hx = half == 0 ? hiX0 : hiX1;
        const uint32_t ly = half == 0 ? loY0 : loY1, hy = half == 0 ? hiY0 : hiY1;
        const uint32_t lz = half == 0 ? loZ0 : loZ1, hz = half == 0 ? hiZ0 : hiZ1;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#ifdef __CUDA_ARCH__
            // near and far plane of an axis as one packed pair: two byte permutes, one
            // packed add, one packed FMA (each lane rounds as the scalar fma_rn does)
            float t0x, t1x, t0y, t1y, t0z, t1z;
            unpack2(fma2(add2(byte_pair(lx, hx, j), kMinus2p23x2), ax2, bx2), t0x, t1x);
            unpack2(fma2(add2(byte_pair(ly, hy, j), kMinus2p23x2), ay2, by2), t0y, t1y);
            unpack2(fma2(add2(byte_pair(lz, hz, j), kMinus2p23x2), az2, bz2), t0z, t1z);
            const float tn = max3(t0x, t0y, fmaxf(t0z, tmin));
            const float tf = min3(t1x, t1y, fminf(t1z, tmax));
#else
            const float t0x = fma_rn(byte_to_float(lx, j), ax, bx);
            const float t1x = fma_rn(byte_to_float(hx, j), ax, bx);
            const float t0y = fma_rn(byte_to_float(ly, j), ay, by);
            const float t1y = fma_rn(byte_to_float(hy, j), ay, by);
            const float t0z = fma_rn(byte_to_float(lz, j), az, bz);
            const float t1z = fma_rn(byte_to_float(hz, j), az, bz);
            const float tn = fmaxf(fmaxf(t0x, t0y), fmaxf(t0z, tmin));
            const float tf = fminf(fminf(t1x, t1y), fminf(t1z, tmax));
#endif
            if (tn <= tf * 1.0000004f)
                hitmask |= ((childBits4 >> (8 * j)) & 7u) << ((bitIndex4 >> (8 * j)) & 31u);
        }
    }
    return hitmask;
}

// Resumable traversal state of one ray: the persistent extend/connect kernels
// keep one per lane and refill a lane with a new ray as soon as its ray ends.
struct Traversal {
    float3 O;
    float3 D;
    float3 invD;
    float tmin;
    float tmax;
    float u;
    float v;
    uint32_t octInv;
    uint32_t hitSlot;
    uint32_t steps;
    uint2 group;
    int sp;
    bool ok;
};

TR_HD void traversal_begin(Traversal& t, const float3& O, const float3& D, float tmin, float tmax, uint32_t root = 0)
{
    const float kTiny = 1e-20f;
    t.O = O;
    t.D = D;
    t.invD = make_float3(1.0f / (fabsf(D.x) > kTiny ? D.x : copysignf(kTiny, D.x)),
                         1.0f / (fabsf(D.y) > kTiny ? D.y : copysignf(kTiny, D.y)),
                         1.0f / (fabsf(D.z) > kTiny ? D.z : copysignf(kTiny, D.z)));
    const uint32_t octant = (t.invD.x < 0.f ? 1u : 0u) | (t.invD.y < 0.f ? 2u : 0u) | (t.invD.z < 0.f ? 4u : 0u);
    t.octInv = 7u - octant;
    t.tmin = tmin;
    t.tmax = tmax;
    t.u = 0.f;
    t.v = 0.f;
    t.hitSlot = 0xffffffffu;
    t.steps = 0;
    t.group = make_uint2(root, 0x80000000u);  // the root as the only internal child of a virtual parent
    t.sp = 0;
    t.ok = true;
}

// One step: the next hit child node of the current group with the leaf
// triangles it reports, then a stack pop if the group is exhausted. Returns
// true when the ray is finished (t.hitSlot, t.tmax, t.u, t.v hold the result;
// t.ok is false if a bound was exceeded).
// The next hit child node of the current group, intersected: the group
// becomes its internal children (the rest of the old group waits on the
// stack); returns its leaf group (base, bits). Returns false when a bound ran
// out (t.ok cleared).
// Node layout a traversal is compiled for: the scene's (a uniform branch per
// node on SceneView::quantNodes), or fixed to fp32 or quantized child boxes.
enum : int { kLayoutScene = 0, kLayoutWide = 1, kLayoutQuant = 2 };

template <bool COUNT, int LAYOUT = kLayoutScene>
TR_HD bool node_step(Traversal& t, uint2* stack, const void* __restrict__ nodes, bool quant, uint32_t stepLimit,
                     TraversalCounts* cnt, uint2& leaves)
{
    leaves = make_uint2(0u, 0u);
    if (t.group.y <= 0x00ffffffu)
        return true;
    const uint32_t hits = t.group.y;
    const uint32_t bit = 31u - clz32(hits);
    t.group.y &= ~(1u << bit);
    const uint32_t slot = (bit - 24u) ^ t.octInv;
    const uint32_t rel = popc32(hits & 0xffu & ((1u << slot) - 1u));
    const uint32_t nodeIx = t.group.x + rel;
    if (t.group.y > 0x00ffffffu) {
        if (t.sp < kTraversalStack)
            stack[t.sp++] = t.group;
        else
            t.ok = false;
    }
    uint32_t childBase, triBase, imask;
    // the node layout is the same for every ray of a launch (a uniform branch
    // when it is not fixed at compile time)
    const bool q = LAYOUT == kLayoutQuant || (LAYOUT == kLayoutScene && quant);
    const uint32_t hm =
        q ? intersect_qnode(static_cast<const QuantNode*>(nodes), nodeIx, t.O, t.invD, t.octInv, t.tmin, t.tmax,
                                childBase, triBase, imask)
              : intersect_wnode(static_cast<const WideNode*>(nodes), nodeIx, t.O, t.invD, t.octInv, t.tmin, t.tmax,
                                childBase, triBase, imask);
    if (COUNT)
        cnt->nodes++;
    t.group = make_uint2(childBase, (hm & 0xff000000u) | imask);
    leaves = make_uint2(triBase, hm & 0x00ffffffu);
    if (++t.steps > stepLimit) {
        t.ok = false;
        return false;
    }
    return true;
}

// Tests the triangles of a leaf group. Returns 2 when an any-hit ray found
// its hit, 1 when a closer hit was recorded, 0 otherwise. PAIR (closest hit
// only) fetches two triangles before testing either.
template <bool ANY, bool COUNT, bool PAIR = false>
TR_HD int leaf_triangles(Traversal& t, uint2 tris, const SceneView& s, TraversalCounts* cnt)
{
    int found = 0;
    auto test = [&](uint32_t slot, const float4& a, const float4& b, const float4& c) -> bool {
        if (COUNT)
            cnt->tris++;
        float tt, uu, vv;
        if (intersect_triangle(t.O, t.D, a, b, c, t.tmin, t.tmax, tt, uu, vv)) {
            if (ANY) {
                t.tmax = tt;
                t.hitSlot = slot;
                return true;
            }
            if (tt < t.tmax || t.hitSlot == 0xffffffffu) {
                t.tmax = tt;
                t.hitSlot = slot;
                t.u = uu;
                t.v = vv;
                found = 1;
            }
        }
        return false;
    };
    if constexpr (ANY || !PAIR) {
        // one triangle at a time (any hit: a second fetch in flight costs the
        // shadow kernel registers and occupancy, and the first hit ends the ray;
        // two-level traversal: it would spill)
        while (tris.y != 0u) {
            const uint32_t k = ffs32(tris.y) - 1u;
            tris.y &= tris.y - 1u;
            const float4* tp = s.bvhTris + 3u * (tris.x + k);
            if (test(tris.x + k, ldg(tp + 0), ldg(tp + 1), ldg(tp + 2)))
                return 2;
        }
        return found;
    } else {
        // closest hit: two triangles per iteration, both fetched before either is
        // tested (the second fetch repeats the first when only one is left); tested
        // in bit order, so the result is that of the one-at-a-time loop
        while (tris.y != 0u) {
            const uint32_t k0 = ffs32(tris.y) - 1u;
            tris.y &= tris.y - 1u;
            const bool two = tris.y != 0u;
            const uint32_t k1 = two ? ffs32(tris.y) - 1u : k0;
            tris.y &= tris.y - 1u;
            const float4* p0 = s.bvhTris + 3u * (tris.x + k0);
            const float4* p1 = s.bvhTris + 3u * (tris.x + k1);
            const float4 a0 = ldg(p0 + 0), b0 = ldg(p0 + 1), c0 = ldg(p0 + 2);
            const float4 a1 = ldg(p1 + 0), b1 = ldg(p1 + 1), c1 = ldg(p1 + 2);
            test(tris.x + k0, a0, b0, c0);
            if (two)
                test(tris.x + k1, a1, b1, c1);
        }
        return found;
    }
}

// One step: the next hit child node of the current group with the leaf
// triangles it reports, then a stack pop if the group is exhausted. Returns
// true when the ray is finished (t.hitSlot, t.tmax, t.u, t.v hold the result;
// t.ok is false if a bound was exceeded).
template <bool ANY, bool COUNT, int LAYOUT = kLayoutScene>
TR_HD bool traversal_step(Traversal& t, uint2* stack, const SceneView& s, TraversalCounts* cnt)
{
    uint2 tris;
    if (!node_step<COUNT, LAYOUT>(t, stack, s.nodes, s.quantNodes != 0, s.stepLimit, cnt, tris))
        return true;
#ifdef __CUDA_ARCH__
    // closest hit: the next node (the first hit child of the new group) into L1
    // while the leaf triangles are tested (extend 51.9 -> 51.6 ms per 1080p,
    // 64 spp heightfield step; shadow rays lost 0.4 ms with it)
    if (!ANY && LAYOUT == kLayoutWide && tris.y != 0u && t.group.y > 0x00ffffffu) {
        const uint32_t hits = t.group.y;
        const uint32_t slot = (31u - clz32(hits) - 24u) ^ t.octInv;
        const uint32_t next = t.group.x + popc32(hits & 0xffu & ((1u << slot) - 1u));
        const char* a = reinterpret_cast<const char*>(static_cast<const WideNode*>(s.nodes) + next);
        asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(a + 128));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(a + 192));
    }
#endif
    if (leaf_triangles<ANY, COUNT, !ANY>(t, tris, s, cnt) == 2)
        return true;
    if (t.group.y <= 0x00ffffffu) {
        if (t.sp == 0)
            return true;
        t.group = stack[--t.sp];
    }
    return false;
}

// Instance transforms applied to a ray: rows (r | t) of the inverse instance
// transform, ((r.x p.x + r.y p.y) + r.z p.z) + t with every operation rounded
// on its own (the oracle applies the same sequence).
TR_HD float3 xform_point(const float4& r0, const float4& r1, const float4& r2, const float3& p)
{
    return make_float3(add_rn(add_rn(add_rn(mul_rn(r0.x, p.x), mul_rn(r0.y, p.y)), mul_rn(r0.z, p.z)), r0.w),
                       add_rn(add_rn(add_rn(mul_rn(r1.x, p.x), mul_rn(r1.y, p.y)), mul_rn(r1.z, p.z)), r1.w),
                       add_rn(add_rn(add_rn(mul_rn(r2.x, p.x), mul_rn(r2.y, p.y)), mul_rn(r2.z, p.z)), r2.w));
}
TR_HD float3 xform_vector(const float4& r0, const float4& r1, const float4& r2, const float3& v)
{
    return make_float3(add_rn(add_rn(mul_rn(r0.x, v.x), mul_rn(r0.y, v.y)), mul_rn(r0.z, v.z)),
                       add_rn(add_rn(mul_rn(r1.x, v.x), mul_rn(r1.y, v.y)), mul_rn(r1.z, v.z)),
                       add_rn(add_rn(mul_rn(r2.x, v.x), mul_rn(r2.y, v.y)), mul_rn(r2.z, v.z)));
}

TR_HD void set_ray(Traversal& t, const float3& O, const float3& D)
{
    const float kTiny = 1e-20f;
    t.O = O;
    t.D = D;
    t.invD = make_float3(1.0f / (fabsf(D.x) > kTiny ? D.x : copysignf(kTiny, D.x)),
                         1.0f / (fabsf(D.y) > kTiny ? D.y : copysignf(kTiny, D.y)),
                         1.0f / (fabsf(D.z) > kTiny ? D.z : copysignf(kTiny, D.z)));
    const uint32_t octant = (t.invD.x < 0.f ? 1u : 0u) | (t.invD.y < 0.f ? 2u : 0u) | (t.invD.z < 0.f ? 4u : 0u);
    t.octInv = 7u - octant;
}

// Two-level traversal (the instance BVH, then the BVH of each instance's mesh
// in object space; replaces OptiX's instance acceleration structure). The
// object-space ray keeps the world ray's parameter t, so t and tmax compare
// across instances.
constexpr uint32_t kNoInstance = 0xffffffffu;

struct TraversalTL {
    Traversal t;          // the current ray (world at the top level, object space inside an instance)
    float3 wO, wD, wInvD;
    uint32_t wOctInv;
    uint32_t inst;        // instance being traversed, kNoInstance at the top level
    int instSp;           // stack depth when it was entered
    uint2 leafGroup;      // top level: instances of a reached leaf group still to enter
    uint32_t hitInst;     // instance of the recorded hit
};

TR_HD void traversal_begin(TraversalTL& r, const float3& O, const float3& D, float tmin, float tmax, uint32_t = 0)
{
    traversal_begin(r.t, O, D, tmin, tmax, 0u);
    r.wO = O;
    r.wD = D;
    r.wInvD = r.t.invD;
    r.wOctInv = r.t.octInv;
    r.inst = kNoInstance;
    r.instSp = -1;
    r.leafGroup = make_uint2(0u, 0u);
    r.hitInst = kNoInstance;
}

// (two levels: the instance BVH has the layout of the mesh BVHs)
template <bool ANY, bool COUNT, int LAYOUT = kLayoutScene>
TR_HD bool traversal_step(TraversalTL& r, uint2* stack, const SceneView& s, TraversalCounts* cnt)
{
    Traversal& t = r.t;
    if (r.inst == kNoInstance && r.leafGroup.y != 0u) {
        // enter the next instance of a top-level leaf group; the rest of the
        // group and the node group being walked wait on the stack
        const uint32_t k = ffs32(r.leafGroup.y) - 1u;
        const uint32_t rest = r.leafGroup.y & (r.leafGroup.y - 1u);
        const uint32_t id = ldg(s.tlasInst + r.leafGroup.x + k);
        const uint32_t need = (t.group.y > 0x00ffffffu ? 1 : 0) + (rest ? 1 : 0);
        if (t.sp + int(need) > kTraversalStack) {
            t.ok = false;
            return true;
        }
        if (t.group.y > 0x00ffffffu)
            stack[t.sp++] = t.group;
        if (rest)
            stack[t.sp++] = make_uint2(r.leafGroup.x, rest);
        r.leafGroup = make_uint2(0u, 0u);
        const float4 r0 = ldg(s.invTransforms + 3u * id + 0u);
        const float4 r1 = ldg(s.invTransforms + 3u * id + 1u);
        const float4 r2 = ldg(s.invTransforms + 3u * id + 2u);
        set_ray(t, xform_point(r0, r1, r2, r.wO), xform_vector(r0, r1, r2, r.wD));
        r.inst = id;
        r.instSp = t.sp;
        t.group = make_uint2(ldg(&s.instInfo[id].x), 0x80000000u);
        if (++t.steps > s.stepLimit) {
            t.ok = false;
            return true;
        }
        return false;
    }
    const bool top = r.inst == kNoInstance;
    uint2 leaves;
    if (!node_step<COUNT, LAYOUT>(t, stack, top ? s.tlasNodes : s.nodes, s.quantNodes != 0, s.stepLimit, cnt,
                                  leaves))
        return true;
    if (top) {
        r.leafGroup = leaves;  // entered one by one in the next steps
    } else {
        const int found = leaf_triangles<ANY, COUNT>(t, leaves, s, cnt);
        if (found)
            r.hitInst = r.inst;
        if (found == 2)
            return true;
    }
    if (t.group.y <= 0x00ffffffu && r.leafGroup.y == 0u) {
        if (r.inst != kNoInstance && t.sp == r.instSp) {
            // the instance is done: back to the world ray at the top level
            t.O = r.wO;
            t.D = r.wD;
            t.invD = r.wInvD;
            t.octInv = r.wOctInv;
            r.inst = kNoInstance;
            r.instSp = -1;
        }
        if (t.sp == 0)
            return true;
        const uint2 e = stack[--t.sp];
        if (r.inst == kNoInstance && e.y <= 0x00ffffffu) {
            r.leafGroup = e;
            t.group = make_uint2(0u, 0u);
        } else {
            t.group = e;
        }
    }
    return false;
}

template <bool TL>
struct TravOf {
    using type = Traversal;
};
template <>
struct TravOf<true> {
    using type = TraversalTL;
};

// The result fields of either traversal.
TR_HD const Traversal& base(const Traversal& t) { return t; }
TR_HD const Traversal& base(const TraversalTL& r) { return r.t; }
TR_HD uint32_t hit_instance(const Traversal&) { return 0u; }
TR_HD uint32_t hit_instance(const TraversalTL& r) { return r.hitInst; }

// Traverses to the end (two levels when the scene has an instance BVH).
// ANY = true stops at the first hit inside [tmin, tmax]. Returns false when a
// bound (stack depth, step count) was exceeded; the hit reported so far is
// kept. COUNT adds the nodes and triangles visited to *cnt.
template <bool ANY, bool COUNT = false>
TR_HD bool traverse(const SceneView& s, const float3& O, const float3& D, float tmin, float& tmax, uint32_t& hitSlot,
                    float& hu, float& hv, TraversalCounts* cnt = nullptr, uint32_t* hitInst = nullptr)
{
    uint2 stack[kTraversalStack];
    if (s.tlasNodes) {
        TraversalTL r;
        traversal_begin(r, O, D, tmin, tmax);
        while (!traversal_step<ANY, COUNT>(r, stack, s, cnt)) {
        }
        tmax = r.t.tmax;
        hitSlot = r.t.hitSlot;
        hu = r.t.u;
        hv = r.t.v;
        if (hitInst)
            *hitInst = r.hitInst;
        return r.t.ok;
    }
    Traversal t;
    traversal_begin(t, O, D, tmin, tmax);
    while (!traversal_step<ANY, COUNT>(t, stack, s, cnt)) {
    }
    tmax = t.tmax;
    hitSlot = t.hitSlot;
    hu = t.u;
    hv = t.v;
    if (hitInst)
        *hitInst = 0u;
    return t.ok;
}

} // namespace tr
