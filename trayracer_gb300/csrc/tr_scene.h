// Host scene flattening: the device records the kernels read, built from a
// tr_scene_desc.
#pragma once

#include <string>
#include <vector>

#include "tr_device.h"

namespace tr {

struct FlatScene {
    std::vector<TriShade> tris;        // by triangle index (two-level: meshes concatenated, object space)
    std::vector<uint32_t> matIdx;      // by triangle index (two-level: mesh material offset added)
    std::vector<uint32_t> meshTriBase; // two-level: first triangle of each mesh
    std::vector<uint32_t> instMesh;    // two-level: mesh of each instance
    std::vector<Material> materials;
    std::vector<TexSlots> texSlots;    // per material when any material has a texture (tex = index + 1)
    std::vector<LightTri> lights;
    std::vector<AliasEntry> alias;
    std::vector<float4> invTransforms; // 3 per instance
    float lightEnergy = 0.f;           // last exclusive prefix (reference LightEnergy)
    float lightEnergyTotal = 0.f;
    float bounds[6] = {0, 0, 0, 0, 0, 0};
};

// Largest texture side accepted.
constexpr uint32_t kMaxTextureSize = 32768;

// Validates the description; returns an empty string when it is usable.
std::string validate_scene(const tr_scene_desc& desc);

// Model::Build (PackedTriangle, Tracer/Resources/Model.cpp:93-167),
// Model::BuildLights (Model.cpp:171-236), Scene::GatherLights
// (Tracer/Renderer/Scene.cpp:275-302) and Material::Property::Build
// (Tracer/Resources/Material.cpp:56-78) for one mesh with one identity
// instance, plus the light alias table.
FlatScene flatten_scene(const tr_scene_desc& desc);

// The mesh of a one-level scene, or mesh i of a two-level one.
inline const tr_mesh_desc& scene_mesh(const tr_scene_desc& d, uint32_t i)
{
    return d.instance_count ? d.meshes[i] : *d.mesh;
}
inline uint32_t scene_mesh_count(const tr_scene_desc& d) { return d.instance_count ? d.mesh_count : 1u; }

// Inverse of an affine 3x4 (rows r.x, r.y, r.z, t), the formula of the
// reference's inverse(float3x4) (Tracer/Utility/LinearMath.h:472-506).
void inverse_3x4(const float* m, float* out);
// R p + t for an instance transform's rows (r | t).
float3 place_point(const float* m, const float3& p);

// Resolves one material as GetIntersectionAttributes does per hit
// (Tracer/CUDA/GPU/CudaMaterial.h:171-183): fp16-rounded properties,
// emissive = Emissive * diffuse, tint and luminance from CIE XYZ.
Material resolve_material(const tr_material_desc& m);

// Walker/Vose alias table over the given weights: small and large work lists
// filled in index order and consumed from the back.
std::vector<AliasEntry> build_alias_table(const std::vector<double>& weights);

float round_to_half(float x);
uint16_t half_bits(float x);

} // namespace tr
