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
    if (!desc.mesh)
        return "scene has no mesh";
    const tr_mesh_desc& m = *desc.mesh;
    if (m.triangle_count > 0 && (!m.positions || !m.indices || !m.material_indices))
        return "mesh arrays missing";
    if (m.triangle_count >= (1u << 31))
        return "too many triangles";
    if (desc.material_count == 0 && m.triangle_count > 0)
        return "scene has no materials";
    if (desc.material_count > 0 && !desc.materials)
        return "material array missing";
    for (uint32_t t = 0; t < m.triangle_count; ++t) {
        for (int k = 0; k < 3; ++k)
            if (m.indices[3 * t + k] >= m.vertex_count)
                return "triangle " + std::to_string(t) + " indexes past the vertex array";
        if (m.material_indices[t] >= desc.material_count)
            return "triangle " + std::to_string(t) + " has an invalid material index";
    }
    for (uint32_t i = 0; i < desc.material_count; ++i)
        if (desc.materials[i].closure > TR_CLOSURE_DISNEY)
            return "material " + std::to_string(i) + " has an unknown closure";
    if (desc.bvh_leaf_size > 3)
        return "bvh_leaf_size must be 0..3";
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

FlatScene flatten_scene(const tr_scene_desc& desc)
{
    FlatScene fs;
    const tr_mesh_desc& m = *desc.mesh;
    const uint32_t n = m.triangle_count;
    fs.tris.resize(n);
    fs.matIdx.resize(n);
    fs.materials.resize(desc.material_count);
    for (uint32_t i = 0; i < desc.material_count; ++i)
        fs.materials[i] = resolve_material(desc.materials[i]);

    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t v = 0; v < m.vertex_count && m.positions; ++v)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::fmin(lo[a], m.positions[3 * v + a]);
            hi[a] = std::fmax(hi[a], m.positions[3 * v + a]);
        }
    for (int a = 0; a < 3; ++a) {
        fs.bounds[a] = lo[a];
        fs.bounds[3 + a] = hi[a];
    }

    auto pos = [&](uint32_t v) { return make_float3(m.positions[3 * v], m.positions[3 * v + 1], m.positions[3 * v + 2]); };
    std::vector<double> energies;
    float sumEnergy = 0.f;
    for (uint32_t t = 0; t < n; ++t) {
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
        TriShade& s = fs.tris[t];
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
        fs.matIdx[t] = m.material_indices[t];

        // emissive triangle -> light (BuildLights + GatherLights, identity instance)
        const tr_material_desc& md = desc.materials[m.material_indices[t]];
        const float3 em = make_float3(md.emissive[0], md.emissive[1], md.emissive[2]);
        if (em.x + em.y + em.z > kEpsilon) {
            LightTri lt{};
            lt.triIx = int32_t(t);
            lt.instIx = 0;
            lt.V0 = v0;
            lt.V1 = v1;
            lt.V2 = v2;
            lt.N = normalize(n0 + n1 + n2);
            const float a = length(v1 - v0), b = length(v2 - v1), c = length(v0 - v2);
            const float sp = (a + b + c) * .5f;
            lt.area = sqrtf(sp * (sp - a) * (sp - b) * (sp - c));
            lt.radiance = em;
            const float3 e = em * lt.area;
            lt.energy = e.x + e.y + e.z;
            lt.N = normalize(lt.N);  // world-space normal of the identity instance
            lt.sumEnergy = sumEnergy;
            sumEnergy += lt.energy;
            fs.lights.push_back(lt);
            energies.push_back(double(lt.energy));
        }
    }
    fs.lightEnergy = fs.lights.empty() ? 0.f : fs.lights.back().sumEnergy;
    fs.lightEnergyTotal = sumEnergy;
    fs.alias = build_alias_table(energies);
    // identity inverse instance transform (rows of a float3x4)
    fs.invTransforms = {make_float4(1, 0, 0, 0), make_float4(0, 1, 0, 0), make_float4(0, 0, 1, 0)};
    return fs;
}

} // namespace tr
