// Host-side run of the 8-wide BVH build + traversal code of the extend/connect
// kernels (tr_trace_host): the same node layouts and the same traversal
// source (one or two levels), compiled for the CPU, so the BVH can be checked
// without a GPU and the traversal work per ray (nodes visited, triangles
// tested) can be counted.
#include <cuda_runtime.h>

#include <thread>
#include <vector>

#include "../../include/trayracer.h"
#include "tr_accel.h"
#include "tr_bvh.h"
#include "tr_scene.h"
#include "tr_traverse.cuh"

using namespace tr;

extern "C" tr_status tr_trace_host(const tr_scene_desc* desc, const float* O4, const float* D4, uint32_t n,
                                   float tmin, int32_t any_hit, uint32_t* hits, uint32_t* counts)
{
    if (!desc || (n && (!O4 || !D4 || !hits)))
        return TR_ERR_INVALID_ARGUMENT;
    if (!validate_scene(*desc).empty())
        return TR_ERR_INVALID_ARGUMENT;
    BvhBuildOptions opt;
    opt.maxLeafSize = desc->bvh_leaf_size ? desc->bvh_leaf_size : 3u;
    opt.threads = desc->build_threads;
    const FlatScene fs = flatten_scene(*desc);
    const SceneAccel acc = build_accel(*desc, fs.meshTriBase, opt);
    const bool quant = (any_hit & 2) != 0;
    any_hit &= 1;
    const std::vector<QuantNode> qnodes = quant ? quantize_nodes(acc.nodes) : std::vector<QuantNode>{};
    const std::vector<QuantNode> qtlas = quant ? quantize_nodes(acc.tlasNodes) : std::vector<QuantNode>{};
    SceneView s{};
    s.nodes = quant ? static_cast<const void*>(qnodes.data()) : static_cast<const void*>(acc.nodes.data());
    s.quantNodes = quant ? 1u : 0u;
    s.bvhTris = acc.tris.data();
    s.nodeCount = uint32_t(acc.nodes.size());
    s.triCount = uint32_t(fs.tris.size());
    s.invTransforms = fs.invTransforms.data();
    if (!acc.tlasNodes.empty()) {
        s.tlasNodes = quant ? static_cast<const void*>(qtlas.data()) : static_cast<const void*>(acc.tlasNodes.data());
        s.tlasInst = acc.tlasInst.data();
        s.instInfo = acc.instInfo.data();
    }

    const unsigned threads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    auto work = [&](unsigned t) {
        for (uint32_t i = t; i < n; i += threads) {
            const float3 O = make_float3(O4[4 * i], O4[4 * i + 1], O4[4 * i + 2]);
            const float3 D = make_float3(D4[4 * i], D4[4 * i + 1], D4[4 * i + 2]);
            float tmax = any_hit ? D4[4 * i + 3] : kDstMax;
            uint32_t slot = 0xffffffffu;
            float u = 0.f, v = 0.f;
            TraversalCounts c{0, 0};
            uint32_t inst = 0;
            if (any_hit)
                traverse<true, true>(s, O, D, tmin, tmax, slot, u, v, &c, &inst);
            else
                traverse<false, true>(s, O, D, tmin, tmax, slot, u, v, &c, &inst);
            uint32_t* h = hits + 4 * size_t(i);
            if (slot != 0xffffffffu) {
                const uint32_t bx = static_cast<uint32_t>(u * 65535.f) & 0xFFFFu;
                const uint32_t by = static_cast<uint32_t>(v * 65535.f) & 0xFFFFu;
                h[0] = (bx << 16) | by;
                h[1] = inst;
                h[2] = f2u(acc.tris[3 * size_t(slot)].w);
                h[3] = f2u(tmax);
            } else {
                h[0] = 0;
                h[1] = 0xffffffffu;
                h[2] = 0xffffffffu;
                h[3] = f2u(kDstMax);
            }
            if (counts) {
                counts[2 * size_t(i)] = c.nodes;
                counts[2 * size_t(i) + 1] = c.tris;
            }
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads; ++t)
        pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool)
        th.join();
    return TR_OK;
}
