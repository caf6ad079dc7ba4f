// Internal interface between the reference kernels compiled as host C++ and
// the harness that drives them (oracle/_ref). TEST INFRASTRUCTURE.
#pragma once

#include "Common/CommonStructs.h"

struct RefSceneBuffers {
    CudaMeshData* meshData;
    CudaMatarial* materials;
    uint32_t* materialOffsets;
    float4* invTransforms;
    uint32_t* modelIndices;
    int32_t lightCount;
    float lightEnergy;
    LightTriangle* lights;
    SkyData* sky;
};

void refk_set_scene(const RefSceneBuffers& b);
void refk_set_frame(const LaunchParams* params, const RayCounters* counters);
void refk_shade(uint32_t pathCount, float4* accumulator, float4* albedo, float4* normals, float4* pathStates,
                uint4* hitData, float4* shadowRays, int resX, int resY, uint32_t stride, uint32_t pathLength,
                uint32_t renderMode, uint32_t renderFlags);

void refo_set_params(const LaunchParams& p);
void refo_launch(uint32_t w, uint32_t h, uint32_t d);

// optixTrace stand-in: closest hit (payload = bary 16:16, instIx, primIx, t bits;
// the miss program zeroes payload 0) or terminate-on-first-hit (payload 0 left
// untouched on a hit, zeroed on a miss).
void ref_host_trace(float3 O, float3 D, float tmin, float tmax, bool anyHit, uint32_t& p0, uint32_t& p1, uint32_t& p2,
                    uint32_t& p3);
