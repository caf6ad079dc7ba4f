// Compiles the reference's path-tracing shade kernel (PathTracingKernel,
// Tracer/CUDA/GPU/Shade/PathTracing.h) and the device globals/setters it reads
// (Tracer/CUDA/GPU/CudaGlobals.h) as host C++, unchanged, from the reference
// tree. TEST INFRASTRUCTURE (oracle/_ref).
#include "host_cuda_shim.h"

uint3 threadIdx, blockIdx, blockDim;

#include "CudaLights.h"
#include "CudaMaterial.h"
#include "Shade/AmbientOcclusion.h"
#include "Shade/AmbientOcclusionShading.h"
#include "Shade/Bitangent.h"
#include "Shade/GeometricNormal.h"
#include "Shade/MaterialID.h"
#include "Shade/MaterialProperty.h"
#include "Shade/ObjectID.h"
#include "Shade/PathTracing.h"
#include "Shade/ShadingNormal.h"
#include "Shade/Tangent.h"
#include "Shade/TextureCoordinate.h"
#include "Shade/Wireframe.h"
#include "Shade/ZDepth.h"

#include "ref_api.h"

void refk_set_scene(const RefSceneBuffers& b)
{
    SetCudaMeshData(b.meshData);
    SetCudaMatarialData(b.materials);
    SetCudaMatarialOffsets(b.materialOffsets);
    SetCudaInvTransforms(b.invTransforms);
    SetCudaModelIndices(b.modelIndices);
    SetCudaLightCount(b.lightCount);
    SetCudaLightEnergy(b.lightEnergy);
    SetCudaLights(b.lights);
    SetCudaSkyData(b.sky);
}

void refk_set_frame(const LaunchParams* params, const RayCounters* counters)
{
    SetCudaLaunchParams(params);
    SetCudaCounters(counters);
}

// Shade(renderMode, ...) of Tracer/CUDA/GPU/cuda.cu:23-85 with the
// <<<ceil(n/128), 128>>> grid walked one thread at a time.
void refk_shade(uint32_t pathCount, float4* accumulator, float4* albedo, float4* normals, float4* pathStates,
                uint4* hitData, float4* shadowRays, int resX, int resY, uint32_t stride, uint32_t pathLength,
                uint32_t renderMode, uint32_t renderFlags)
{
    blockDim = make_uint3(128, 1, 1);
    const uint32_t blocks = (pathCount + 127) / 128;
    for (uint32_t b = 0; b < blocks; ++b) {
        blockIdx = make_uint3(b, 0, 0);
        for (uint32_t t = 0; t < 128; ++t) {
            threadIdx = make_uint3(t, 0, 0);
#define REF_ARGS pathCount, accumulator, albedo, normals, pathStates, hitData, shadowRays, resX, resY, stride, \
                 pathLength, renderFlags
            switch (static_cast<RenderModes>(renderMode)) {
            case RenderModes::AmbientOcclusion: AmbientOcclusionKernel(REF_ARGS); break;
            case RenderModes::AmbientOcclusionShading: AmbientOcclusionShadingKernel(REF_ARGS); break;
            case RenderModes::Bitangent: BitangentKernel(REF_ARGS); break;
            case RenderModes::GeometricNormal: GeometricNormalKernel(REF_ARGS); break;
            case RenderModes::MaterialID: MaterialIDKernel(REF_ARGS); break;
            case RenderModes::MaterialProperty: MaterialPropertyKernel(REF_ARGS); break;
            case RenderModes::ObjectID: ObjectIDKernel(REF_ARGS); break;
            case RenderModes::PathTracing: PathTracingKernel(REF_ARGS); break;
            case RenderModes::ShadingNormal: ShadingNormalKernel(REF_ARGS); break;
            case RenderModes::Tangent: TangentKernel(REF_ARGS); break;
            case RenderModes::TextureCoordinate: TextureCoordinateKernel(REF_ARGS); break;
            case RenderModes::Wireframe: WireframeKernel(REF_ARGS); break;
            case RenderModes::ZDepth: ZDepthKernel(REF_ARGS); break;
            default: break;
            }
#undef REF_ARGS
        }
    }
}

// One closure of the reference (Lambert.h:53-59, Diffuse.h:36-42, Disney.h:573-579) on explicit inputs.
// in: wo[3], wi[3], T[3], then HitMaterial fields in declaration order (CudaMaterial.h:31-52):
//     diffuse[3], metallic, emissive[3], subsurface, tint[3], specular, roughness, specularTint,
//     anisotropic, sheen, sheenTint, clearcoat, clearcoatGloss, luminance, then r0, r1.
// out: extend.T[3], extend.pdf, extend.wi[3], extend.flags, shadow.T[3], shadow.pdf.
extern "C" void ref_closure(int type, const float* in, float* out)
{
    ShadingInfo info{};
    info.wo = make_float3(in[0], in[1], in[2]);
    info.wi = make_float3(in[3], in[4], in[5]);
    info.T = make_float3(in[6], in[7], in[8]);
    HitMaterial m{};
    const float* q = in + 9;
    m.diffuse = make_float3(q[0], q[1], q[2]);
    m.metallic = q[3];
    m.emissive = make_float3(q[4], q[5], q[6]);
    m.subsurface = q[7];
    m.tint = make_float3(q[8], q[9], q[10]);
    m.specular = q[11];
    m.roughness = q[12];
    m.specularTint = q[13];
    m.anisotropic = q[14];
    m.sheen = q[15];
    m.sheenTint = q[16];
    m.clearcoat = q[17];
    m.clearcoatGloss = q[18];
    m.luminance = q[19];
    const float r0 = q[20], r1 = q[21];
    Closure c{};
    if (type == 2)
        c = DisneyClosure(info, m, r0, r1);
    else if (type == 1)
        c = DiffuseClosure(info, m, r0, r1);
    else
        c = LambertClosure(info, m, r0, r1);
    const float o[14] = {c.extend.T.x, c.extend.T.y, c.extend.T.z, c.extend.pdf, c.extend.wi.x, c.extend.wi.y,
                         c.extend.wi.z, __uint_as_float(c.extend.flags), c.shadow.T.x, c.shadow.T.y, c.shadow.T.z,
                         c.shadow.pdf, 0.f, 0.f};
    std::memcpy(out, o, sizeof(o));
}

// tea<2>(v0, v1) followed by n rnd() draws of thirdparty/CUDA/random.h.
extern "C" void ref_rng(uint32_t v0, uint32_t v1, uint32_t n, float* out)
{
    uint32_t seed = tea<2>(v0, v1);
    for (uint32_t i = 0; i < n; ++i)
        out[i] = rnd(seed);
}
