// Host BVH builder: binned-SAH binary BVH, collapsed into an 8-wide BVH with
// the compressed wide BVH's child and leaf encoding (fp32 or 8-bit quantized
// child boxes) for the extend/connect kernels. Replaces the OptiX
// acceleration-structure build of the reference (Model::Upload,
// Tracer/Resources/Model.cpp:240-306; OptixRenderer::BuildAccel,
// Tracer/Optix/OptixRenderer.cpp:90-123).
#pragma once

#include <cstdint>
#include <vector>

#include "tr_device.h"

namespace tr {

struct Aabb {
    float lo[3];
    float hi[3];
};

struct BinaryNode {
    Aabb box;
    uint32_t left;     // internal: index of the left child (right = left + 1); leaf: first primitive ref
    uint32_t count;    // 0 = internal, else primitives in the leaf
};

struct BvhBuildOptions {
    uint32_t maxLeafSize = 3;   // 1..3 (the CWBVH leaf encoding holds up to 3)
    // true: the binary BVH is built down to one triangle per leaf and the wide leaves
    // (up to maxLeafSize triangles) are chosen by the SAH-optimal collapse
    bool sahCollapse = true;
    uint32_t bins = 16;
    uint32_t threads = 0;       // 0 = hardware concurrency
};

struct BinaryBvh {
    std::vector<BinaryNode> nodes;
    std::vector<uint32_t> primRefs;   // leaf ranges index this array; values are triangle indices
};

struct Cwbvh {
    std::vector<WideNode> nodes;
    std::vector<float4> tris;          // 3 float4 per triangle slot
    std::vector<uint32_t> triPrim;     // triangle index per slot
};

// Builds a binary BVH over triangles given as positions (float3 per vertex)
// (leaves of up to maxLeafSize triangles, or of one when sahCollapse)
// and indices (uint3 per triangle).
BinaryBvh build_binary_bvh(const float* positions, const uint32_t* indices, uint32_t triCount,
                           const BvhBuildOptions& options);

// Builds a binary BVH over axis-aligned boxes (the instances of a two-level
// scene).
BinaryBvh build_binary_bvh_boxes(const Aabb* boxes, uint32_t count, const BvhBuildOptions& options);

// Collapses a binary BVH into 8-wide nodes (fp32 child boxes) and packs the
// traversal triangles (v0, e1 = v1 - v0, e2 = v2 - v0). positions == nullptr
// (a BVH over boxes): no triangles, triPrim names the primitive of each leaf
// slot. sahMaxLeaf = 0: greedy collapse (open the largest internal child until
// 8); 1..3: SAH-optimal collapse with leaves of up to sahMaxLeaf triangles.
Cwbvh collapse_to_cwbvh(const BinaryBvh& bvh, const float* positions, const uint32_t* indices,
                        uint32_t sahMaxLeaf = 0);

// The same nodes with 8-bit quantized child boxes (rounded outwards against
// each node's box, the union of its children's).
std::vector<QuantNode> quantize_nodes(const std::vector<WideNode>& nodes);

// Node layout of an uploaded BVH: mode 0 (auto) keeps fp32 child boxes while the
// nodes fit kWideNodeBudget (they then stay in L2 beside the wavefront
// buffers) and the scene has one level (the two-level traversal holds more
// state, and fp32 nodes make it spill), 1 always fp32, 2 always quantized.
// Returns true for quantized.
constexpr size_t kWideNodeBudget = size_t(64) << 20;
inline bool quantized_nodes(size_t nodeCount, uint32_t mode, bool twoLevel = false)
{
    return mode == 2u || (mode == 0u && (twoLevel || nodeCount * sizeof(WideNode) > kWideNodeBudget));
}

} // namespace tr

namespace tr {
// The 8-wide BVH of one mesh as the options ask: binary build, then the
// SAH-optimal or the greedy collapse.
Cwbvh build_cwbvh(const float* positions, const uint32_t* indices, uint32_t triCount, const BvhBuildOptions& opt,
                  Aabb* bounds = nullptr);
}  // namespace tr
