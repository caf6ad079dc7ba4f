// Harness around the reference's kernels compiled as host C++ (oracle/_ref):
// builds the reference's device structures for a tr_scene_desc and runs the
// reference's frame loop (DeviceRenderer::RenderFrame / RenderBounce,
// Tracer/Renderer/DeviceRenderer.cpp:97-274) on one host thread, with
// optixTrace served by the oracle's traversal. TEST INFRASTRUCTURE.
#include "host_cuda_shim.h"
#include "ref_api.h"

#include "CUDA/helper_math.h"

#include "../oracle.h"

#include <vector>

namespace {

struct RefCtx {
    orc_scene* orc = nullptr;
    std::vector<PackedTriangle> tris;
    std::vector<uint32_t> matIdx;
    std::vector<CudaMatarial> mats;
    std::vector<LightTriangle> lights;
    CudaMeshData mesh{};
    uint32_t materialOffsets[1] = {0};
    uint32_t modelIndices[1] = {0};
    float4 invTransforms[3];
    SkyData sky{};
    LaunchParams lp{};
    RayCounters counters{};
};

RefCtx* g_ctx = nullptr;

float3 f3n(float x, float y, float z) { return make_float3(x, y, z); }
float3 nrm(float3 v)
{
    const float l = 1.0f / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    return make_float3(v.x * l, v.y * l, v.z * l);
}

// Material::Property::Build (Tracer/Resources/Material.cpp:56-78) with the
// property kinds of Material::Material (Material.cpp:102-114).
CudaMaterialProperty prop(float r, float g, float b, uint8_t channels, uint8_t useTexture)
{
    CudaMaterialProperty p{};
    p.textureMap = 0;
    p.r = __float2half(r);
    p.g = __float2half(g);
    p.b = __float2half(b);
    p.colorChannels = channels;
    p.useTexture = useTexture;
    return p;
}

void set_frame_params(RefCtx* c, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H,
                      uint32_t sampleCount, float4* acc, float4* states, uint4* hits, float4* shadow)
{
    LaunchParams& lp = c->lp;
    lp = LaunchParams{};
    lp.resX = W;
    lp.resY = H;
    lp.sampleCount = sampleCount;
    lp.accumulator = acc;
    lp.cameraPos = f3n(cam->position[0], cam->position[1], cam->position[2]);
    lp.cameraSide = f3n(cam->side[0], cam->side[1], cam->side[2]);
    lp.cameraUp = f3n(cam->up[0], cam->up[1], cam->up[2]);
    lp.cameraForward = f3n(cam->forward[0], cam->forward[1], cam->forward[2]);
    lp.cameraAperture = cam->aperture;
    lp.cameraDistortion = cam->distortion;
    lp.cameraFocalDist = cam->focal_dist;
    lp.cameraFov = cam->fov;
    lp.cameraBokehSideCount = cam->bokeh_side_count;
    lp.cameraBokehRotation = cam->bokeh_rotation;
    lp.pathStates = states;
    lp.hitData = hits;
    lp.shadowRays = shadow;
    lp.renderMode = RenderModes::PathTracing;
    lp.kernelSettings.multiSample = st->multi_sample;
    lp.kernelSettings.maxDepth = st->max_depth;
    lp.kernelSettings.seed = st->seed;
    lp.kernelSettings.aoDist = 1.f;
    lp.kernelSettings.zDepthMax = 1.f;
    lp.kernelSettings.rayEpsilon = st->ray_epsilon;
    g_ctx = c;
    refk_set_frame(&c->lp, &c->counters);
}

} // namespace

void ref_host_trace(float3 O, float3 D, float tmin, float tmax, bool anyHit, uint32_t& p0, uint32_t& p1,
                    uint32_t& p2, uint32_t& p3)
{
    const float o[3] = {O.x, O.y, O.z}, d[3] = {D.x, D.y, D.z};
    uint32_t prim = 0;
    float t = 0, u = 0, v = 0;
    const int hit = orc_trace_ray(g_ctx->orc, o, d, tmin, tmax, anyHit ? 1 : 0, &prim, &t, &u, &v);
    if (anyHit) {
        if (!hit)
            p0 = 0;
        return;
    }
    if (!hit) {
        p0 = 0;
        return;
    }
    const uint32_t bx = static_cast<uint32_t>(u * 65535.f) & 0xFFFF;
    const uint32_t by = static_cast<uint32_t>(v * 65535.f) & 0xFFFF;
    p0 = (bx << 16) | by;
    p1 = 0;
    p2 = prim;
    p3 = __float_as_uint(t);
}

extern "C" {

void* ref_create(const tr_scene_desc* desc)
{
    if (!desc || !desc->mesh)
        return nullptr;
    RefCtx* c = new RefCtx();
    c->orc = orc_scene_create(desc);
    const tr_mesh_desc& m = *desc->mesh;
    const uint32_t n = m.triangle_count;
    c->tris.resize(n);
    c->matIdx.assign(m.material_indices, m.material_indices + n);
    float sumEnergy = 0;
    for (uint32_t t = 0; t < n; ++t) {
        const uint32_t ix[3] = {m.indices[3 * t], m.indices[3 * t + 1], m.indices[3 * t + 2]};
        float3 p[3], nn[3];
        float2 uv[3];
        for (int k = 0; k < 3; ++k) {
            p[k] = f3n(m.positions[3 * ix[k]], m.positions[3 * ix[k] + 1], m.positions[3 * ix[k] + 2]);
            uv[k] = m.texcoords ? make_float2(m.texcoords[2 * ix[k]], m.texcoords[2 * ix[k] + 1]) : make_float2(0, 0);
        }
        for (int k = 0; k < 3; ++k)
            nn[k] = m.normals ? f3n(m.normals[3 * ix[k]], m.normals[3 * ix[k] + 1], m.normals[3 * ix[k] + 2])
                              : nrm(cross(p[1] - p[0], p[2] - p[0]));
        // Model::Build, Tracer/Resources/Model.cpp:105-163
        PackedTriangle& q = c->tris[t];
        q.v0x = p[0].x; q.v0y = p[0].y; q.v0z = p[0].z;
        q.v1x = p[1].x; q.v1y = p[1].y; q.v1z = p[1].z;
        q.v2x = p[2].x; q.v2y = p[2].y; q.v2z = p[2].z;
        q.uv0x = __float2half(uv[0].x); q.uv0y = __float2half(uv[0].y);
        q.uv1x = __float2half(uv[1].x); q.uv1y = __float2half(uv[1].y);
        q.uv2x = __float2half(uv[2].x); q.uv2y = __float2half(uv[2].y);
        q.N0x = __float2half(nn[0].x); q.N0y = __float2half(nn[0].y); q.N0z = __float2half(nn[0].z);
        q.N1x = __float2half(nn[1].x); q.N1y = __float2half(nn[1].y); q.N1z = __float2half(nn[1].z);
        q.N2x = __float2half(nn[2].x); q.N2y = __float2half(nn[2].y); q.N2z = __float2half(nn[2].z);
        const float3 N = normalize(nn[0] + nn[1] + nn[2]);
        q.Nx = __float2half(N.x); q.Ny = __float2half(N.y); q.Nz = __float2half(N.z);
        // Model::BuildLights (Model.cpp:205-230) + Scene::GatherLights (Scene.cpp:283-297)
        const tr_material_desc& md = desc->materials[m.material_indices[t]];
        const float3 em = f3n(md.emissive[0], md.emissive[1], md.emissive[2]);
        if (em.x + em.y + em.z > 1e-3f) {
            LightTriangle lt{};
            lt.triIx = int32_t(t);
            lt.V0 = p[0];
            lt.V1 = p[1];
            lt.V2 = p[2];
            lt.N = normalize(normalize(nn[0] + nn[1] + nn[2]));
            const float a = length(lt.V1 - lt.V0), b = length(lt.V2 - lt.V1), cc = length(lt.V0 - lt.V2);
            const float s = (a + b + cc) * .5f;
            lt.area = sqrtf(s * (s - a) * (s - b) * (s - cc));
            lt.radiance = em;
            const float3 e = em * lt.area;
            lt.energy = e.x + e.y + e.z;
            lt.sumEnergy = sumEnergy;
            lt.instIx = 0;
            sumEnergy += lt.energy;
            c->lights.push_back(lt);
        }
    }
    c->mats.resize(desc->material_count);
    for (uint32_t i = 0; i < desc->material_count; ++i) {
        const tr_material_desc& d = desc->materials[i];
        CudaMatarial& cm = c->mats[i];
        auto f = [&](MaterialPropertyIds id, float v) { cm.properties[size_t(id)] = prop(v, 0.f, 0.f, 1, 1); };
        f(MaterialPropertyIds::Anisotropic, d.anisotropic);
        f(MaterialPropertyIds::Clearcoat, d.clearcoat);
        f(MaterialPropertyIds::ClearcoatGloss, d.clearcoat_gloss);
        cm.properties[size_t(MaterialPropertyIds::Diffuse)] = prop(d.diffuse[0], d.diffuse[1], d.diffuse[2], 3, 1);
        cm.properties[size_t(MaterialPropertyIds::Emissive)] = prop(d.emissive[0], d.emissive[1], d.emissive[2], 3, 0);
        f(MaterialPropertyIds::Metallic, d.metallic);
        cm.properties[size_t(MaterialPropertyIds::Normal)] = prop(0.f, 0.f, 0.f, 0, 1);
        f(MaterialPropertyIds::Roughness, d.roughness);
        f(MaterialPropertyIds::Sheen, d.sheen);
        f(MaterialPropertyIds::SheenTint, d.sheen_tint);
        f(MaterialPropertyIds::Specular, d.specular);
        f(MaterialPropertyIds::SpecularTint, d.specular_tint);
        f(MaterialPropertyIds::Subsurface, d.subsurface);
    }
    c->mesh.triangles = c->tris.data();
    c->mesh.materialIndices = c->matIdx.data();
    // inverse of the identity instance transform, as float3x4 rows (Renderer.cpp:482-484)
    c->invTransforms[0] = make_float4(1, 0, 0, 0);
    c->invTransforms[1] = make_float4(0, 1, 0, 0);
    c->invTransforms[2] = make_float4(0, 0, 1, 0);
    c->sky.skyEnabled = 0;
    c->sky.drawSun = 0;
    return c;
}

void ref_destroy(void* ctx)
{
    RefCtx* c = static_cast<RefCtx*>(ctx);
    if (!c)
        return;
    orc_scene_destroy(c->orc);
    delete c;
}

static void bind_scene(RefCtx* c)
{
    RefSceneBuffers b;
    b.meshData = &c->mesh;
    b.materials = c->mats.data();
    b.materialOffsets = c->materialOffsets;
    b.invTransforms = c->invTransforms;
    b.modelIndices = c->modelIndices;
    b.lightCount = int32_t(c->lights.size());
    // SetCudaLightEnergy(lightData.back().sumEnergy), Renderer.cpp:500
    b.lightEnergy = c->lights.empty() ? 0.f : c->lights.back().sumEnergy;
    b.lights = c->lights.data();
    b.sky = &c->sky;
    refk_set_scene(b);
    g_ctx = c;
}

// Primary raygen: InitializeFilm + camera ray + closest hit for W x H x ms paths.
void ref_primary(void* ctx, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H,
                 uint32_t sampleCount, float* states, uint32_t* hits, float* accumulator)
{
    RefCtx* c = static_cast<RefCtx*>(ctx);
    bind_scene(c);
    set_frame_params(c, cam, st, W, H, sampleCount, reinterpret_cast<float4*>(accumulator),
                     reinterpret_cast<float4*>(states), reinterpret_cast<uint4*>(hits), nullptr);
    c->lp.rayGenMode = RayGenModes::Primary;
    refo_set_params(c->lp);
    refo_launch(W, H, st->multi_sample);
}

void ref_secondary(void* ctx, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H,
                   uint32_t sampleCount, uint32_t pathCount, float* states, uint32_t* hits)
{
    RefCtx* c = static_cast<RefCtx*>(ctx);
    bind_scene(c);
    set_frame_params(c, cam, st, W, H, sampleCount, nullptr, reinterpret_cast<float4*>(states),
                     reinterpret_cast<uint4*>(hits), nullptr);
    c->lp.rayGenMode = RayGenModes::Secondary;
    refo_set_params(c->lp);
    refo_launch(pathCount, 1, 1);
}

// PathTracingKernel over pathCount jobs; counters[0..1] = extend, shadow rays written.
void ref_shade(void* ctx, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H,
               uint32_t sampleCount, uint32_t pathLength, uint32_t pathCount, float* states, uint32_t* hits,
               float* shadow, float* accumulator, float* albedo, float* normals, uint32_t* counters)
{
    RefCtx* c = static_cast<RefCtx*>(ctx);
    bind_scene(c);
    set_frame_params(c, cam, st, W, H, sampleCount, reinterpret_cast<float4*>(accumulator),
                     reinterpret_cast<float4*>(states), reinterpret_cast<uint4*>(hits),
                     reinterpret_cast<float4*>(shadow));
    c->counters = RayCounters{};
    const uint32_t stride = W * H * st->multi_sample;
    refk_shade(pathCount, reinterpret_cast<float4*>(accumulator), reinterpret_cast<float4*>(albedo),
               reinterpret_cast<float4*>(normals), reinterpret_cast<float4*>(states), reinterpret_cast<uint4*>(hits),
               reinterpret_cast<float4*>(shadow), int(W), int(H), stride, pathLength);
    counters[0] = c->counters.extendRays;
    counters[1] = c->counters.shadowRays;
}

void ref_shadow(void* ctx, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H,
                uint32_t sampleCount, uint32_t shadowCount, float* shadow, float* accumulator)
{
    RefCtx* c = static_cast<RefCtx*>(ctx);
    bind_scene(c);
    set_frame_params(c, cam, st, W, H, sampleCount, reinterpret_cast<float4*>(accumulator), nullptr, nullptr,
                     reinterpret_cast<float4*>(shadow));
    c->lp.rayGenMode = RayGenModes::Shadow;
    refo_set_params(c->lp);
    refo_launch(shadowCount, 1, 1);
}

// DeviceRenderer::RenderFrame (DeviceRenderer.cpp:97-133) for one frame:
// accumulator in/out (float4 per pixel); ext/shadow ray counts per bounce.
void ref_render_frame(void* ctx, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H,
                      uint32_t sampleCount, float* accumulator, uint32_t* extCounts, uint32_t* shCounts)
{
    RefCtx* c = static_cast<RefCtx*>(ctx);
    const uint32_t stride = W * H * st->multi_sample;
    std::vector<float4> states(3 * size_t(stride)), shadow(3 * size_t(stride)), albedo(W * H), normals(W * H);
    std::vector<uint4> hits(stride);
    uint32_t pathCount = stride;
    uint32_t pathLength = 0;
    for (uint32_t b = 0; b < st->max_depth; ++b) {
        extCounts[b] = 0;
        shCounts[b] = 0;
    }
    do {
        if (pathLength == 0)
            ref_primary(ctx, cam, st, W, H, sampleCount, &states[0].x, &hits[0].x, accumulator);
        else
            ref_secondary(ctx, cam, st, W, H, sampleCount, pathCount, &states[0].x, &hits[0].x);
        extCounts[pathLength] = pathCount;
        uint32_t counters[2];
        ref_shade(ctx, cam, st, W, H, sampleCount, pathLength, pathCount, &states[0].x, &hits[0].x, &shadow[0].x,
                  accumulator, &albedo[0].x, &normals[0].x, counters);
        pathCount = counters[0];
        if (counters[1] > 0) {
            ref_shadow(ctx, cam, st, W, H, sampleCount, counters[1], &shadow[0].x, accumulator);
            shCounts[pathLength] = counters[1];
        }
    } while (++pathLength < st->max_depth && pathCount > 0);
    (void)c;
}

} // extern "C"
