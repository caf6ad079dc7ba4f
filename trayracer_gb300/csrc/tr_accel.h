// Acceleration structures of a scene on the host: one 8-wide BVH per mesh
// (concatenated, indices rebased) and, for two-level scenes, one over the
// instances (replaces the OptiX GAS/IAS builds of Model::Upload,
// Tracer/Resources/Model.cpp:240-306, and OptixRenderer::BuildAccel,
// Tracer/Optix/OptixRenderer.cpp:90-123).
#pragma once

#include <vector>

#include "tr_bvh.h"
#include "tr_scene.h"

namespace tr {

struct SceneAccel {
    std::vector<WideNode> nodes;      // every mesh's BVH, child and triangle bases rebased
    std::vector<float4> tris;          // traversal triangles; v0.w = the mesh's own triangle index
    std::vector<uint32_t> meshRoot;    // first node of each mesh's BVH
    std::vector<WideNode> tlasNodes;  // two-level scenes: BVH over the instances' world boxes
    std::vector<uint32_t> tlasInst;    // instance of each leaf slot of tlasNodes
    std::vector<uint2> instInfo;       // per instance: (BVH root node, first triangle of its mesh)
};

// meshTriBase: first triangle of each mesh in the concatenated shading
// records (FlatScene::meshTriBase). One-level scenes: the single mesh's BVH at
// node 0, no instance level.
SceneAccel build_accel(const tr_scene_desc& desc, const std::vector<uint32_t>& meshTriBase,
                       const BvhBuildOptions& opt);

} // namespace tr
