// Host stand-ins for the CUDA device built-ins the reference's shading headers
// use, so those headers compile unchanged as host C++ (oracle/_ref).
// TEST INFRASTRUCTURE: part of the oracle; never linked into the product.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

// device min/max overloads for float (helper_math.h's host fallbacks only cover int)
static inline float min(float a, float b) { return fminf(a, b); }
static inline float max(float a, float b) { return fmaxf(a, b); }
static inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
static inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }

static inline uint32_t __float_as_uint(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint_as_float(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline int __float_as_int(float f) { int u; std::memcpy(&u, &f, 4); return u; }
static inline float __saturatef(float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }
static inline void __threadfence() {}
// kernels run one job at a time on one host thread
static inline uint32_t atomicAdd(uint32_t* p, uint32_t v) { const uint32_t o = *p; *p = o + v; return o; }
// tex2D<float4>: texture object = texture index + 1 of the bound scene, sampled as the
// device does (bilinear, wrap, normalised coordinates), by the oracle's sampler
void ref_tex2d(cudaTextureObject_t t, float x, float y, float* out);
template <class T> static inline T tex2D(cudaTextureObject_t t, float x, float y)
{
    float o[4];
    ref_tex2d(t, x, y, o);
    return T{o[0], o[1], o[2], o[3]};
}

#undef __launch_bounds__
#define __launch_bounds__(...)
// __constant__ / __device__ symbols become host globals; setters copy into them
#define cudaMemcpyToSymbol(sym, src, n) std::memcpy((void*)&(sym), (src), (n))
