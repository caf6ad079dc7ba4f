// Random streams of the path tracer.
//
// RefRng reproduces the reference's streams: a two-round TEA hash seeds a
// 24-bit LCG (thirdparty/CUDA/random.h:31-67), keyed as in
// Tracer/Optix/GPU/optix.cu:247 (camera) and
// Tracer/CUDA/GPU/Shade/PathTracing.h:103 (shading).
//
// CounterRng is the default: every draw is a pure function of
// (pixel, sample, bounce, dimension, frame seed), computed with the pcg4d hash
// of Jarzynski and Olano ("Hash Functions for GPU Rendering", JCGT 9(3),
// 2020). Dimension d of a bounce uses word d & 3 of
// pcg4d(pixel, sample, bounce << 8 | d >> 2, seed); draws are consumed in
// order, so a path's sequence does not depend on how the wavefront scheduled it.
#pragma once

#include "tr_vec.h"

namespace tr {

TR_HD uint32_t tea2(uint32_t v0, uint32_t v1)
{
    uint32_t s0 = 0;
    for (int n = 0; n < 2; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

struct RefRng {
    uint32_t state;
    TR_HD float next()
    {
        state = 1664525u * state + 1013904223u;
        return float(state & 0x00FFFFFFu) / float(0x01000000);
    }
};

TR_HD uint4 pcg4d(uint4 v)
{
    v.x = v.x * 1664525u + 1013904223u;
    v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u;
    v.w = v.w * 1664525u + 1013904223u;
    v.x += v.y * v.w;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    v.w += v.y * v.z;
    v.x ^= v.x >> 16;
    v.y ^= v.y >> 16;
    v.z ^= v.z >> 16;
    v.w ^= v.w >> 16;
    v.x += v.y * v.w;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    v.w += v.y * v.z;
    return v;
}

struct CounterRng {
    uint32_t pixel, sample, bounce, seed;
    uint32_t dim;
    uint4 block;
    TR_HD void init(uint32_t p, uint32_t s, uint32_t b, uint32_t sd)
    {
        pixel = p;
        sample = s;
        bounce = b;
        seed = sd;
        dim = 0;
    }
    TR_HD float next()
    {
        if ((dim & 3u) == 0)
            block = pcg4d(make_uint4(pixel, sample, (bounce << 8) | (dim >> 2), seed));
        const uint32_t w = (dim & 3u) == 0 ? block.x : (dim & 3u) == 1 ? block.y : (dim & 3u) == 2 ? block.z : block.w;
        ++dim;
        return float(w >> 8) * (1.0f / 16777216.0f);
    }
};

} // namespace tr
