// Compiles the reference's OptiX programs (Tracer/Optix/GPU/optix.cu: camera
// ray generation, Primary/Secondary/Shadow raygen, closest-hit/miss payloads)
// as host C++, unchanged, from the reference tree. optixTrace is served by the
// oracle's host traversal (same fp32 triangle test as the GPU kernels).
// TEST INFRASTRUCTURE (oracle/_ref).
#include "host_cuda_shim.h"

#include "optix7/optix.h"

#include "ref_api.h"

static uint3 g_launchIndex, g_launchDims;
static inline uint3 optixGetLaunchIndex() { return g_launchIndex; }
static inline uint3 optixGetLaunchDimensions() { return g_launchDims; }
static inline void optixTrace(OptixTraversableHandle, float3 O, float3 D, float tmin, float tmax, float,
                              OptixVisibilityMask, unsigned flags, unsigned, unsigned, unsigned, uint32_t& p0,
                              uint32_t& p1, uint32_t& p2, uint32_t& p3)
{
    ref_host_trace(O, D, tmin, tmax, (flags & OPTIX_RAY_FLAG_TERMINATE_ON_FIRST_HIT) != 0, p0, p1, p2, p3);
}
// the hit programs' payload writes are done by ref_host_trace
static inline float2 optixGetTriangleBarycentrics() { return make_float2(0, 0); }
static inline unsigned optixGetInstanceIndex() { return 0; }
static inline unsigned optixGetPrimitiveIndex() { return 0; }
static inline float optixGetRayTmax() { return 0; }
static inline void optixTerminateRay() {}
static inline void optixSetPayload_0(unsigned) {}
static inline void optixSetPayload_1(unsigned) {}
static inline void optixSetPayload_2(unsigned) {}
static inline void optixSetPayload_3(unsigned) {}

#include "Optix/GPU/optix.cu"

void refo_set_params(const LaunchParams& p) { params = p; }

// optixLaunch(w, h, d) of the raygen program, one launch index at a time
void refo_launch(uint32_t w, uint32_t h, uint32_t d)
{
    g_launchDims = make_uint3(w, h, d);
    for (uint32_t z = 0; z < d; ++z)
        for (uint32_t y = 0; y < h; ++y)
            for (uint32_t x = 0; x < w; ++x) {
                g_launchIndex = make_uint3(x, y, z);
                __raygen__();
            }
}
