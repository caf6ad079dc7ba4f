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
    std::vector<std::vector<PackedTriangle>> tris;   // per model
    std::vector<std::vector<uint32_t>> matIdx;       // per model
    std::vector<CudaMatarial> mats;
    std::vector<LightTriangle> lights;
    std::vector<CudaMeshData> meshData;              // per instance (Renderer.cpp:473-486)
    std::vector<uint32_t> materialOffsets;           // per model
    std::vector<uint32_t> modelIndices;              // per instance
    std::vector<float4> invTransforms;               // 3 per instance
    SkyData sky{};
    LaunchParams lp{};
    RayCounters counters{};
};

RefCtx* g_ctx = nullptr;

// render mode of the next frames (DeviceRenderer::RenderFrame's renderMode / renderFlags)
uint32_t g_renderMode = uint32_t(RenderModes::PathTracing);
uint32_t g_renderFlags = 0;
float g_aoDist = 1.f, g_zDepthMax = 1.f;

// The reference's float3x4 (Tracer/Utility/LinearMath.h:205-210: float3 x; tx; y; ty; z; tz)
// with its inverse (:472-506) and transform (:274-281), restated here because that
// header's host intrinsics collide with this shim's.
struct M34 {
    float3 x; float tx;
    float3 y; float ty;
    float3 z; float tz;
};
M34 m34_inverse(const M34& a)
{
    const float det3 = a.x.x * (a.y.y * a.z.z - a.y.z * a.z.y) - a.x.y * (a.y.x * a.z.z - a.y.z * a.z.x) +
                       a.x.z * (a.y.x * a.z.y - a.y.y * a.z.x);
    const float inv_det3 = 1.0f / det3;
    const float i00 = inv_det3 * (a.y.y * a.z.z - a.z.y * a.y.z);
    const float i01 = inv_det3 * (a.x.z * a.z.y - a.z.z * a.x.y);
    const float i02 = inv_det3 * (a.x.y * a.y.z - a.y.y * a.x.z);
    const float i10 = inv_det3 * (a.y.z * a.z.x - a.z.z * a.y.x);
    const float i11 = inv_det3 * (a.x.x * a.z.z - a.z.x * a.x.z);
    const float i12 = inv_det3 * (a.x.z * a.y.x - a.y.z * a.x.x);
    const float i20 = inv_det3 * (a.y.x * a.z.y - a.z.x * a.y.y);
    const float i21 = inv_det3 * (a.x.y * a.z.x - a.z.y * a.x.x);
    const float i22 = inv_det3 * (a.x.x * a.y.y - a.y.x * a.x.y);
    M34 r;
    r.x = make_float3(i00, i01, i02);
    r.y = make_float3(i10, i11, i12);
    r.z = make_float3(i20, i21, i22);
    r.tx = -i00 * a.tx - i01 * a.ty - i02 * a.tz;
    r.ty = -i10 * a.tx - i11 * a.ty - i12 * a.tz;
    r.tz = -i20 * a.tx - i21 * a.ty - i22 * a.tz;
    return r;
}
float4 m34_transform(const M34& a, const float4& b)
{
    return make_float4(dot(b, make_float4(a.x.x, a.y.x, a.z.x, a.tx)), dot(b, make_float4(a.x.y, a.y.y, a.z.y, a.ty)),
                       dot(b, make_float4(a.x.z, a.y.z, a.z.z, a.tz)), b.w);
}

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
    lp.renderMode = static_cast<RenderModes>(g_renderMode);
    lp.renderFlags = g_renderFlags;
    lp.kernelSettings.multiSample = st->multi_sample;
    lp.kernelSettings.maxDepth = st->max_depth;
    lp.kernelSettings.seed = st->seed;
    lp.kernelSettings.aoDist = g_aoDist;
    lp.kernelSettings.zDepthMax = g_zDepthMax;
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
    uint32_t inst = 0;
    const int hit = orc_trace_ray(g_ctx->orc, o, d, tmin, tmax, anyHit ? 1 : 0, &prim, &t, &u, &v, &inst);
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
    p1 = inst;
    p2 = prim;
    p3 = __float_as_uint(t);
}

void ref_tex2d(cudaTextureObject_t t, float x, float y, float* out)
{
    orc_texture_sample(g_ctx->orc, uint32_t(t - 1u), x, y, out);
}

extern "C" {

void ref_set_render_mode(uint32_t mode, uint32_t flags, float aoDist, float zDepthMax)
{
    g_renderMode = mode;
    g_renderFlags = flags;
    g_aoDist = aoDist;
    g_zDepthMax = zDepthMax;
}

void* ref_create(const tr_scene_desc* desc)
{
    if (!desc || (desc->instance_count ? !desc->meshes || !desc->instances : !desc->mesh))
        return nullptr;
    RefCtx* c = new RefCtx();
    c->orc = orc_scene_create(desc);
    const bool twoLevel = desc->instance_count > 0;
    const uint32_t models = twoLevel ? desc->mesh_count : 1u;
    c->tris.resize(models);
    c->matIdx.resize(models);
    for (uint32_t mi = 0; mi < models; ++mi) {
        const tr_mesh_desc& m = twoLevel ? desc->meshes[mi] : *desc->mesh;
        const uint32_t n = m.triangle_count;
        c->tris[mi].resize(n);
        c->matIdx[mi].assign(m.material_indices, m.material_indices + n);
        c->materialOffsets.push_back(twoLevel && desc->mesh_material_offsets ? desc->mesh_material_offsets[mi] : 0u);
        for (uint32_t t = 0; t < n; ++t) {
            const uint32_t ix[3] = {m.indices[3 * t], m.indices[3 * t + 1], m.indices[3 * t + 2]};
            float3 p[3], nn[3];
            float2 uv[3];
            for (int k = 0; k < 3; ++k) {
                p[k] = f3n(m.positions[3 * ix[k]], m.positions[3 * ix[k] + 1], m.positions[3 * ix[k] + 2]);
                uv[k] = m.texcoords ? make_float2(m.texcoords[2 * ix[k]], m.texcoords[2 * ix[k] + 1])
                                    : make_float2(0, 0);
            }
            for (int k = 0; k < 3; ++k)
                nn[k] = m.normals ? f3n(m.normals[3 * ix[k]], m.normals[3 * ix[k] + 1], m.normals[3 * ix[k] + 2])
                                  : nrm(cross(p[1] - p[0], p[2] - p[0]));
            // Model::Build, Tracer/Resources/Model.cpp:105-163
            PackedTriangle& q = c->tris[mi][t];
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
        }
    }
    // instances: mesh data, model index, inverse transform (Renderer.cpp:473-486), then the
    // lights of each instance (Model::BuildLights, Model.cpp:205-230; Scene::GatherLights,
    // Scene.cpp:283-297)
    float sumEnergy = 0;
    const uint32_t instances = twoLevel ? desc->instance_count : 1u;
    for (uint32_t i = 0; i < instances; ++i) {
        const uint32_t mi = twoLevel ? desc->instances[i].mesh : 0u;
        M34 xf{make_float3(1, 0, 0), 0, make_float3(0, 1, 0), 0, make_float3(0, 0, 1), 0};
        if (twoLevel)
            std::memcpy(&xf, desc->instances[i].transform, sizeof(xf));
        const M34 inv = m34_inverse(xf);
        float rows[12];
        std::memcpy(rows, &inv, sizeof(rows));
        for (int r = 0; r < 3; ++r)
            c->invTransforms.push_back(make_float4(rows[4 * r], rows[4 * r + 1], rows[4 * r + 2], rows[4 * r + 3]));
        c->modelIndices.push_back(mi);
        CudaMeshData md{};
        md.triangles = c->tris[mi].data();
        md.materialIndices = c->matIdx[mi].data();
        c->meshData.push_back(md);
        const tr_mesh_desc& m = twoLevel ? desc->meshes[mi] : *desc->mesh;
        for (uint32_t t = 0; t < m.triangle_count; ++t) {
            const tr_material_desc& md2 = desc->materials[m.material_indices[t] + c->materialOffsets[mi]];
            const float3 em = f3n(md2.emissive[0], md2.emissive[1], md2.emissive[2]);
            if (!(em.x + em.y + em.z > 1e-3f))
                continue;
            const PackedTriangle& q = c->tris[mi][t];
            const float3 p0 = f3n(q.v0x, q.v0y, q.v0z), p1 = f3n(q.v1x, q.v1y, q.v1z), p2 = f3n(q.v2x, q.v2y, q.v2z);
            const uint32_t ix[3] = {m.indices[3 * t], m.indices[3 * t + 1], m.indices[3 * t + 2]};
            float3 nn[3];
            for (int k = 0; k < 3; ++k)
                nn[k] = m.normals ? f3n(m.normals[3 * ix[k]], m.normals[3 * ix[k] + 1], m.normals[3 * ix[k] + 2])
                                  : nrm(cross(p1 - p0, p2 - p0));
            LightTriangle lt{};
            lt.triIx = int32_t(t);
            lt.V0 = p0;
            lt.V1 = p1;
            lt.V2 = p2;
            lt.N = normalize(normalize(nn[0] + nn[1] + nn[2]));
            const float a = length(lt.V1 - lt.V0), b = length(lt.V2 - lt.V1), cc = length(lt.V0 - lt.V2);
            const float s = (a + b + cc) * .5f;
            lt.area = sqrtf(s * (s - a) * (s - b) * (s - cc));
            lt.radiance = em;
            const float3 e = em * lt.area;
            lt.energy = e.x + e.y + e.z;
            if (twoLevel) {
                // GatherLights: the reference's transform(float3x4, float4) (LinearMath.h:274-281)
                lt.V0 = make_float3(m34_transform(xf, make_float4(lt.V0, 1)));
                lt.V1 = make_float3(m34_transform(xf, make_float4(lt.V1, 1)));
                lt.V2 = make_float3(m34_transform(xf, make_float4(lt.V2, 1)));
                lt.N = normalize(make_float3(m34_transform(xf, make_float4(lt.N, 0))));
            }
            lt.sumEnergy = sumEnergy;
            lt.instIx = int32_t(i);
            sumEnergy += lt.energy;
            c->lights.push_back(lt);
        }
    }
    c->mats.resize(desc->material_count);
    for (uint32_t i = 0; i < desc->material_count; ++i) {
        const tr_material_desc& d = desc->materials[i];
        CudaMatarial& cm = c->mats[i];
        // Material::Property::Build (Material.cpp:56-78): textureMap = the texture object
        // (here its index + 1) where the property has a texture
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
        if (desc->material_textures && desc->texture_count > 0)
            for (uint32_t p = 0; p < TR_PROP_COUNT; ++p) {
                const uint32_t ti = desc->material_textures[size_t(i) * TR_PROP_COUNT + p];
                if (ti != TR_NO_TEXTURE)
                    cm.properties[p].textureMap = cudaTextureObject_t(ti) + 1u;
            }
    }
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
    b.meshData = c->meshData.data();
    b.materials = c->mats.data();
    b.materialOffsets = c->materialOffsets.data();
    b.invTransforms = c->invTransforms.data();
    b.modelIndices = c->modelIndices.data();
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
               reinterpret_cast<float4*>(shadow), int(W), int(H), stride, pathLength, g_renderMode, g_renderFlags);
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

// Sky::SetSunDir / SetTurbidity / Build (Sky.cpp): the SkyData the reference's SampleSky
// reads (NULL: disabled, as a context starts).
void ref_set_sky(void* ctx, const tr_sky_desc* sky)
{
    RefCtx* c = static_cast<RefCtx*>(ctx);
    c->sky = SkyData{};
    if (!sky)
        return;
    const float3 dir = normalize(make_float3(sky->sun_dir[0], sky->sun_dir[1], sky->sun_dir[2]));
    constexpr float Pi = 3.1415926535897932f;  // LinearMath.h:16
    const float diameter = sky->sun_angular_diameter * Pi / (60.f * 180.f);
    const float radius = diameter * .5f;
    c->sky.sunDir = dir;
    c->sky.skyEnabled = sky->enabled ? 1 : 0;
    c->sky.drawSun = sky->draw_sun ? 1.f : 0.f;
    c->sky.sunArea = Pi * radius * radius;
    c->sky.cosSunAngularDiameter = cosf(diameter);
    c->sky.sunIntensity = sky->sun_intensity;
    c->sky.turbidity = clamp(sky->turbidity, 1.f, 10.f);
    c->sky.selectionBias = sky->selection_bias;
    c->sky.sunEnergy = sky->enabled ? sky->sun_intensity * sky->selection_bias : 0.f;
}

// DeviceRenderer::PickRay (DeviceRenderer.cpp:71-92): the RayPick raygen (optix.cu:345-377) for
// one pixel; out = the RayPickResult's 9 words.
void ref_pick_ray(void* ctx, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H, int32_t x,
                  int32_t y, float* out)
{
    RefCtx* c = static_cast<RefCtx*>(ctx);
    bind_scene(c);
    set_frame_params(c, cam, st, W, H, 0, nullptr, nullptr, nullptr, nullptr);
    RayPickResult r{};
    c->lp.rayGenMode = RayGenModes::RayPick;
    c->lp.rayPickPixel = make_int2(x, y);
    c->lp.rayPickResult = &r;
    refo_set_params(c->lp);
    refo_launch(1, 1, 1);
    c->lp.rayPickResult = nullptr;
    static_assert(sizeof(RayPickResult) == 9 * sizeof(float), "RayPickResult is 9 words");
    std::memcpy(out, &r, sizeof(r));
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
