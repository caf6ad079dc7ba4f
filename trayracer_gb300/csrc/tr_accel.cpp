// Host acceleration-structure build of a scene; see tr_accel.h.
#include "tr_accel.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace tr {

SceneAccel build_accel(const tr_scene_desc& desc, const std::vector<uint32_t>& meshTriBase,
                       const BvhBuildOptions& opt)
{
    SceneAccel out;
    const bool twoLevel = desc.instance_count > 0;
    const uint32_t meshCount = scene_mesh_count(desc);
    std::vector<Aabb> meshBox(meshCount);
    for (uint32_t mi = 0; mi < meshCount; ++mi) {
        const tr_mesh_desc& m = scene_mesh(desc, mi);
        const Cwbvh wide = build_cwbvh(m.positions, m.indices, m.triangle_count, opt, &meshBox[mi]);
        const uint32_t nodeBase = uint32_t(out.nodes.size());
        const uint32_t slotBase = uint32_t(out.tris.size() / 3);
        out.meshRoot.push_back(nodeBase);
        for (WideNode n : wide.nodes) {
            n.hdr.x += nodeBase;
            n.hdr.y += slotBase;
            out.nodes.push_back(n);
        }
        out.tris.insert(out.tris.end(), wide.tris.begin(), wide.tris.end());
    }
    if (!twoLevel)
        return out;

    // instance level: world boxes of the placed mesh boxes, slightly widened so
    // that rounding of the placement never culls a hit found in object space
    std::vector<Aabb> boxes;
    std::vector<uint32_t> ids;
    for (uint32_t i = 0; i < desc.instance_count; ++i) {
        const uint32_t mi = desc.instances[i].mesh;
        out.instInfo.push_back(make_uint2(out.meshRoot[mi], meshTriBase[mi]));
        const Aabb& b = meshBox[mi];
        if (!(b.lo[0] <= b.hi[0]))
            continue;  // empty mesh
        Aabb w;
        for (int a = 0; a < 3; ++a) {
            w.lo[a] = INFINITY;
            w.hi[a] = -INFINITY;
        }
        for (int c = 0; c < 8; ++c) {
            const float3 p = place_point(desc.instances[i].transform,
                                         make_float3((c & 1) ? b.hi[0] : b.lo[0], (c & 2) ? b.hi[1] : b.lo[1],
                                                     (c & 4) ? b.hi[2] : b.lo[2]));
            const float q[3] = {p.x, p.y, p.z};
            for (int a = 0; a < 3; ++a) {
                w.lo[a] = std::min(w.lo[a], q[a]);
                w.hi[a] = std::max(w.hi[a], q[a]);
            }
        }
        float ext = 0.f;
        for (int a = 0; a < 3; ++a)
            ext = std::max(ext, std::max(std::fabs(w.lo[a]), std::fabs(w.hi[a])));
        const float pad = ext * 1e-6f + 1e-30f;
        for (int a = 0; a < 3; ++a) {
            w.lo[a] -= pad;
            w.hi[a] += pad;
        }
        boxes.push_back(w);
        ids.push_back(i);
    }
    BvhBuildOptions topOpt = opt;
    topOpt.maxLeafSize = 1;
    const BinaryBvh top = build_binary_bvh_boxes(boxes.data(), uint32_t(boxes.size()), topOpt);
    const Cwbvh wideTop = collapse_to_cwbvh(top, nullptr, nullptr);
    out.tlasNodes = wideTop.nodes;
    out.tlasInst.reserve(wideTop.triPrim.size());
    for (uint32_t p : wideTop.triPrim)
        out.tlasInst.push_back(ids[p]);
    return out;
}

} // namespace tr
