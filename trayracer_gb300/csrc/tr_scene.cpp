// Host scene flattening for the wavefront kernels.
#include "tr_scene.h"

#include <cuda_fp16.h>

#include <cmath>
#include <cstring>

namespace tr {

uint16_t half_bits(float x)
{
    const __half h = __float2half(x);
    const __half_raw r = h;
    return r.x;
}

float round_to_half(float x)
{
    __half_raw r;
    r.x = half_bits(x);
    return __half2float(__half(r));
}

std::string validate_scene(const tr_scene_desc& desc)
{
    if (desc.instance_count) {
        if (!desc.meshes || !desc.instances || desc.mesh_count == 0)
            return "two-level scene without meshes or instances";
        for (uint32_t i = 0; i < desc.instance_count; ++i)
            if (desc.instances[i].mesh >= desc.mesh_count)
                return "instance " + std::to_string(i) + " names a missing mesh";
    } else if (!desc.mesh) {
        return "scene has no mesh";
    }
    if (desc.material_count > 0 && !desc.materials)
        return "material array missing";
    uint64_t total = 0;
    for (uint32_t mi = 0; mi < scene_mesh_count(desc); ++mi) {
        const tr_mesh_desc& m = scene_mesh(desc, mi);
        const uint32_t offset = desc.instance_count && desc.mesh_material_offsets ? desc.mesh_material_offsets[mi] : 0u;
        if (m.triangle_count > 0 && (!m.positions || !m.indices || !m.material_indices))
            return "mesh arrays missing";
        total += m.triangle_count;
        if (total >= (1u << 31))
            return "too many triangles";
        if (desc.material_count == 0 && m.triangle_count > 0)
            return "scene has no materials";
        for (uint32_t t = 0; t < m.triangle_count; ++t) {
            for (int k = 0; k < 3; ++k)
                if (m.indices[3 * t + k] >= m.vertex_count)
                    return "triangle " + std::to_string(t) + " indexes past the vertex array";
            if (uint64_t(m.material_indices[t]) + offset >= desc.material_count)
                return "triangle " + std::to_string(t) + " has an invalid material index";
        }
    }
    for (uint32_t i = 0; i < desc.material_count; ++i)
        if (desc.materials[i].closure > TR_CLOSURE_DISNEY)
            return "material " + std::to_string(i) + " has an unknown closure";
    if (desc.bvh_leaf_size > 3)
        return "bvh_leaf_size must be 0..3";
    if (desc.texture_count > 0 && !desc.textures)
        return "texture array missing";
    for (uint32_t i = 0; i < desc.texture_count; ++i) {
        const tr_texture_desc& t = desc.textures[i];
        if (t.width == 0 || t.height == 0 || t.width > kMaxTextureSize || t.height > kMaxTextureSize || !t.texels)
            return "texture " + std::to_string(i) + " must have texels and a size in [1, 32768]";
    }
    if (desc.material_textures) {
        for (uint32_t i = 0; i < desc.material_count; ++i)
            for (uint32_t p = 0; p < TR_PROP_COUNT; ++p) {
                const uint32_t ti = desc.material_textures[size_t(i) * TR_PROP_COUNT + p];
                if (ti == TR_NO_TEXTURE)
                    continue;
                if (ti >= desc.texture_count)
                    return "material " + std::to_string(i) + " names a missing texture";
                if (p == TR_PROP_EMISSIVE)
                    return "material " + std::to_string(i) + ": the emissive property takes no texture";
            }
    }
    return std::string();
}

Material resolve_material(const tr_material_desc& d)
{
    Material m{};
    m.diffuse = make_float3(round_to_half(d.diffuse[0]), round_to_half(d.diffuse[1]), round_to_half(d.diffuse[2]));
    const float3 tintXYZ = linear_to_xyz(m.diffuse);
    m.metallic = round_to_half(d.metallic);
    const float3 em = make_float3(round_to_half(d.emissive[0]), round_to_half(d.emissive[1]), round_to_half(d.emissive[2]));
    m.emissive = em * m.diffuse;
    m.subsurface = round_to_half(d.subsurface);
    m.tint = tintXYZ.y > 0 ? xyz_to_linear(tintXYZ * (1.f / tintXYZ.y)) : f3(1.f);
    m.specular = round_to_half(d.specular);
    m.roughness = round_to_half(d.roughness);
    m.specularTint = round_to_half(d.specular_tint);
    m.anisotropic = round_to_half(d.anisotropic);
    m.sheen = round_to_half(d.sheen);
    m.sheenTint = round_to_half(d.sheen_tint);
    m.clearcoat = round_to_half(d.clearcoat);
    m.clearcoatGloss = round_to_half(d.clearcoat_gloss);
    m.luminance = tintXYZ.y;
    m.closure = d.closure;
    m.isEmissive = (m.emissive.x + m.emissive.y + m.emissive.z > kEpsilon) ? 1u : 0u;
    return m;
}

std::vector<AliasEntry> build_alias_table(const std::vector<double>& weights)
{
    const size_t n = weights.size();
    std::vector<AliasEntry> table(n);
    if (n == 0)
        return table;
    double total = 0.0;
    for (double w : weights)
        total += w;
    std::vector<double> scaled(n);
    std::vector<uint32_t> small, large;
    small.reserve(n);
    large.reserve(n);
    for (size_t i = 0; i < n; ++i) {
        scaled[i] = total > 0.0 ? weights[i] * double(n) / total : 1.0;
        if (scaled[i] < 1.0)
            small.push_back(uint32_t(i));
        else
            large.push_back(uint32_t(i));
    }
    while (!small.empty() && !large.empty()) {
        const uint32_t s = small.back();
        small.pop_back();
        const uint32_t l = large.back();
        large.pop_back();
        table[s].prob = float(scaled[s]);
        table[s].alias = l;
        scaled[l] = (scaled[l] + scaled[s]) - 1.0;
        if (scaled[l] < 1.0)
            small.push_back(l);
        else
            large.push_back(l);
    }
    for (uint32_t l : large) {
        table[l].prob = 1.0f;
        table[l].alias = l;
    }
    for (uint32_t s : small) {
        table[s].prob = 1.0f;
        table[s].alias = s;
    }
    return table;
}

void inverse_3x4(const float* m, float* out)
{
    // rows (x | tx), (y | ty), (z | tz); LinearMath.h:472-506
    const float xx = m[0], xy = m[1], xz = m[2], tx = m[3];
    const float yx = m[4], yy = m[5], yz = m[6], ty = m[7];
    const float zx = m[8], zy = m[9], zz = m[10], tz = m[11];
    const float det3 = xx * (yy * zz - yz * zy) - xy * (yx * zz - yz * zx) + xz * (yx * zy - yy * zx);
    const float inv = 1.0f / det3;
    const float i00 = inv * (yy * zz - zy * yz), i01 = inv * (xz * zy - zz * xy), i02 = inv * (xy * yz - yy * xz);
    const float i10 = inv * (yz * zx - zz * yx), i11 = inv * (xx * zz - zx * xz), i12 = inv * (xz * yx - yz * xx);
    const float i20 = inv * (yx * zy - zx * yy), i21 = inv * (xy * zx - zy * xx), i22 = inv * (xx * yy - yx * xy);
    out[0] = i00; out[1] = i01; out[2] = i02; out[3] = -i00 * tx - i01 * ty - i02 * tz;
    out[4] = i10; out[5] = i11; out[6] = i12; out[7] = -i10 * tx - i11 * ty - i12 * tz;
    out[8] = i20; out[9] = i21; out[10] = i22; out[11] = -i20 * tx - i21 * ty - i22 * tz;
}

// p' = R p + t for the rows (r | t) of an instance transform; the order of the
// operations is shared with the oracle so both place lights identically.
float3 place_point(const float* m, const float3& p)
{
    return make_float3(((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3], ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
                       ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]);
}

namespace {

// normal transform with the inverse rows, as the shading code applies them
// (CudaMaterial.h:204-211: transform(tx, ty, tz, n) = inverse^T n)
float3 place_normal(const float* inv, const float3& n)
{
    return make_float3((n.x * inv[0] + n.y * inv[4]) + n.z * inv[8], (n.x * inv[1] + n.y * inv[5]) + n.z * inv[9],
                       (n.x * inv[2] + n.y * inv[6]) + n.z * inv[10]);
}

} // namespace

FlatScene flatten_scene(const tr_scene_desc& desc)
{
    FlatScene fs;
    fs.materials.resize(desc.material_count);
    for (uint32_t i = 0; i < desc.material_count; ++i)
        fs.materials[i] = resolve_material(desc.materials[i]);
    // textures per material (texture index + 1 until the upload puts the texture objects in)
    if (desc.material_textures && desc.texture_count > 0) {
        fs.texSlots.assign(desc.material_count, TexSlots{});
        bool any = false;
        for (uint32_t i = 0; i < desc.material_count; ++i) {
            TexSlots& ts = fs.texSlots[i];
            for (uint32_t p = 0; p < TR_PROP_COUNT; ++p) {
                const uint32_t ti = desc.material_textures[size_t(i) * TR_PROP_COUNT + p];
                if (ti != TR_NO_TEXTURE) {
                    ts.tex[p] = uint64_t(ti) + 1u;
                    fs.materials[i].texMask |= 1u << p;
                    any = true;
                }
            }
            for (int k = 0; k < 3; ++k)
                ts.emissive[k] = round_to_half(desc.materials[i].emissive[k]);
        }
        if (!any)
            fs.texSlots.clear();
    }
    const bool twoLevel = desc.instance_count > 0;
    const uint32_t meshCount = scene_mesh_count(desc);

    // shading records of every mesh, object space (Model::Build, Model.cpp:93-167)
    uint32_t total = 0;
    for (uint32_t mi = 0; mi < meshCount; ++mi) {
        fs.meshTriBase.push_back(total);
        total += scene_mesh(desc, mi).triangle_count;
    }
    fs.tris.resize(total);
    fs.matIdx.resize(total);
    for (uint32_t mi = 0; mi < meshCount; ++mi) {
        const tr_mesh_desc& m = scene_mesh(desc, mi);
        const uint32_t base = fs.meshTriBase[mi];
        const uint32_t offset = twoLevel && desc.mesh_material_offsets ? desc.mesh_material_offsets[mi] : 0u;
        auto pos = [&](uint32_t v) {
            return make_float3(m.positions[3 * v], m.positions[3 * v + 1], m.positions[3 * v + 2]);
        };
        for (uint32_t t = 0; t < m.triangle_count; ++t) {
            const uint32_t i0 = m.indices[3 * t], i1 = m.indices[3 * t + 1], i2 = m.indices[3 * t + 2];
            const float3 v0 = pos(i0), v1 = pos(i1), v2 = pos(i2);
            float3 n0, n1, n2;
            if (m.normals) {
                n0 = make_float3(m.normals[3 * i0], m.normals[3 * i0 + 1], m.normals[3 * i0 + 2]);
                n1 = make_float3(m.normals[3 * i1], m.normals[3 * i1 + 1], m.normals[3 * i1 + 2]);
                n2 = make_float3(m.normals[3 * i2], m.normals[3 * i2 + 1], m.normals[3 * i2 + 2]);
            } else {
                n0 = n1 = n2 = normalize(cross(v1 - v0, v2 - v0));
            }
            float2 t0 = make_float2(0.f, 0.f), t1 = t0, t2 = t0;
            if (m.texcoords) {
                t0 = make_float2(m.texcoords[2 * i0], m.texcoords[2 * i0 + 1]);
                t1 = make_float2(m.texcoords[2 * i1], m.texcoords[2 * i1 + 1]);
                t2 = make_float2(m.texcoords[2 * i2], m.texcoords[2 * i2 + 1]);
            }
            TriShade& s = fs.tris[base + t];
            s.v0x = v0.x; s.v0y = v0.y; s.v0z = v0.z;
            s.v1x = v1.x; s.v1y = v1.y; s.v1z = v1.z;
            s.v2x = v2.x; s.v2y = v2.y; s.v2z = v2.z;
            s.uv0x = half_bits(t0.x); s.uv0y = half_bits(t0.y);
            s.uv1x = half_bits(t1.x); s.uv1y = half_bits(t1.y);
            s.uv2x = half_bits(t2.x); s.uv2y = half_bits(t2.y);
            s.N0x = half_bits(n0.x); s.N0y = half_bits(n0.y); s.N0z = half_bits(n0.z);
            s.N1x = half_bits(n1.x); s.N1y = half_bits(n1.y); s.N1z = half_bits(n1.z);
            s.N2x = half_bits(n2.x); s.N2y = half_bits(n2.y); s.N2z = half_bits(n2.z);
            const float3 N = normalize(n0 + n1 + n2);
            s.Nx = half_bits(N.x); s.Ny = half_bits(N.y); s.Nz = half_bits(N.z);
            fs.matIdx[base + t] = m.material_indices[t] + offset;
        }
    }

    // instances: inverse transforms, world bounds, lights in instance then
    // triangle order (Scene::GatherLights, Scene.cpp:275-302; Model::BuildLights,
    // Model.cpp:171-236: Heron area in object space, N = normalize(N0 + N1 + N2))
    const float identity[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    const uint32_t instCount = twoLevel ? desc.instance_count : 1u;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    std::vector<double> energies;
    float sumEnergy = 0.f;
    for (uint32_t i = 0; i < instCount; ++i) {
        const uint32_t mi = twoLevel ? desc.instances[i].mesh : 0u;
        const float* xf = twoLevel ? desc.instances[i].transform : identity;
        float inv[12];
        if (twoLevel)
            inverse_3x4(xf, inv);
        else
            std::copy(identity, identity + 12, inv);
        fs.instMesh.push_back(mi);
        for (int r = 0; r < 3; ++r)
            fs.invTransforms.push_back(make_float4(inv[4 * r], inv[4 * r + 1], inv[4 * r + 2], inv[4 * r + 3]));
        const tr_mesh_desc& m = scene_mesh(desc, mi);
        auto pos = [&](uint32_t v) {
            return make_float3(m.positions[3 * v], m.positions[3 * v + 1], m.positions[3 * v + 2]);
        };
        for (uint32_t v = 0; v < m.vertex_count && m.positions; ++v) {
            const float3 p = twoLevel ? place_point(xf, pos(v)) : pos(v);
            const float c[3] = {p.x, p.y, p.z};
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::fmin(lo[a], c[a]);
                hi[a] = std::fmax(hi[a], c[a]);
            }
        }
        for (uint32_t t = 0; t < m.triangle_count; ++t) {
            const tr_material_desc& md = desc.materials[fs.matIdx[fs.meshTriBase[mi] + t]];
            const float3 em = make_float3(md.emissive[0], md.emissive[1], md.emissive[2]);
            if (!(em.x + em.y + em.z > kEpsilon))
                continue;
            const uint32_t i0 = m.indices[3 * t], i1 = m.indices[3 * t + 1], i2 = m.indices[3 * t + 2];
            const float3 v0 = pos(i0), v1 = pos(i1), v2 = pos(i2);
            float3 n0, n1, n2;
            if (m.normals) {
                n0 = make_float3(m.normals[3 * i0], m.normals[3 * i0 + 1], m.normals[3 * i0 + 2]);
                n1 = make_float3(m.normals[3 * i1], m.normals[3 * i1 + 1], m.normals[3 * i1 + 2]);
                n2 = make_float3(m.normals[3 * i2], m.normals[3 * i2 + 1], m.normals[3 * i2 + 2]);
            } else {
                n0 = n1 = n2 = normalize(cross(v1 - v0, v2 - v0));
            }
            LightTri lt{};
            lt.triIx = int32_t(fs.meshTriBase[mi] + t);  // global triangle index (its material: matIdx[triIx])
            lt.instIx = int32_t(i);
            lt.V0 = twoLevel ? place_point(xf, v0) : v0;
            lt.V1 = twoLevel ? place_point(xf, v1) : v1;
            lt.V2 = twoLevel ? place_point(xf, v2) : v2;
            const float3 N = normalize(n0 + n1 + n2);
            lt.N = twoLevel ? normalize(place_normal(inv, normalize(N))) : N;
            const float a = length(v1 - v0), b = length(v2 - v1), c = length(v0 - v2);
            const float sp = (a + b + c) * .5f;
            lt.area = sqrtf(sp * (sp - a) * (sp - b) * (sp - c));
            lt.radiance = em;
            const float3 e = em * lt.area;
            lt.energy = e.x + e.y + e.z;
            lt.N = normalize(lt.N);
            lt.sumEnergy = sumEnergy;
            sumEnergy += lt.energy;
            fs.lights.push_back(lt);
            energies.push_back(double(lt.energy));
        }
    }
    for (int a = 0; a < 3; ++a) {
        fs.bounds[a] = lo[a];
        fs.bounds[3 + a] = hi[a];
    }
    fs.lightEnergy = fs.lights.empty() ? 0.f : fs.lights.back().sumEnergy;
    fs.lightEnergyTotal = sumEnergy;
    fs.alias = build_alias_table(energies);
    return fs;
}

} // namespace tr
