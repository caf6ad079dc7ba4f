// Host BVH builder: binned SAH over triangle bounds, then a collapse (SAH-optimal
// or greedy) to an 8-wide BVH with the child and leaf encoding of the compressed
// wide BVH (octant-ordered child slots; Ylitie, Karras, Laine, HPG 2017), its
// child boxes in fp32 (WideNode) and, for BVHs too large for L2, quantized to 8
// bits (QuantNode, quantize_nodes).
#include "tr_bvh.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>

namespace tr {
namespace {

struct PrimInfo {
    float lo[3];
    float hi[3];
    float c[3];
};

inline void box_empty(Aabb& b)
{
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = INFINITY;
        b.hi[a] = -INFINITY;
    }
}
inline void box_grow(Aabb& b, const float* lo, const float* hi)
{
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = std::min(b.lo[a], lo[a]);
        b.hi[a] = std::max(b.hi[a], hi[a]);
    }
}
inline float box_area(const Aabb& b)
{
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    if (!(dx >= 0.f) || !(dy >= 0.f) || !(dz >= 0.f))
        return 0.f;
    return 2.f * (dx * dy + dy * dz + dz * dx);
}

struct BinaryBuilder {
    const std::vector<PrimInfo>& prims;
    std::vector<uint32_t>& refs;
    std::vector<BinaryNode>& nodes;
    BvhBuildOptions opt;
    std::atomic<uint32_t> nodeCount{1};
    std::atomic<int> threadsLeft{0};

    BinaryBuilder(const std::vector<PrimInfo>& p, std::vector<uint32_t>& r, std::vector<BinaryNode>& n,
                  const BvhBuildOptions& o)
        : prims(p), refs(r), nodes(n), opt(o)
    {
    }

    void make_leaf(uint32_t nodeIx, uint32_t begin, uint32_t end, const Aabb& box)
    {
        BinaryNode& n = nodes[nodeIx];
        n.box = box;
        n.left = begin;
        n.count = end - begin;
    }

    void build(uint32_t nodeIx, uint32_t begin, uint32_t end)
    {
        const uint32_t count = end - begin;
        Aabb box, cbox;
        box_empty(box);
        box_empty(cbox);
        for (uint32_t i = begin; i < end; ++i) {
            const PrimInfo& p = prims[refs[i]];
            box_grow(box, p.lo, p.hi);
            box_grow(cbox, p.c, p.c);
        }
        if (count == 1) {
            make_leaf(nodeIx, begin, end, box);
            return;
        }

        // binned SAH over all three axes
        const uint32_t B = std::max(2u, std::min(opt.bins, 64u));
        float bestCost = INFINITY;
        int bestAxis = -1;
        uint32_t bestSplit = 0;
        const float parentArea = box_area(box);
        for (int axis = 0; axis < 3; ++axis) {
            const float extent = cbox.hi[axis] - cbox.lo[axis];
            if (!(extent > 0.f))
                continue;
            Aabb binBox[64];
            uint32_t binCount[64];
            for (uint32_t b = 0; b < B; ++b) {
                box_empty(binBox[b]);
                binCount[b] = 0;
            }
            const float k = float(B) / extent;
            for (uint32_t i = begin; i < end; ++i) {
                const PrimInfo& p = prims[refs[i]];
                uint32_t b = uint32_t((p.c[axis] - cbox.lo[axis]) * k);
                b = std::min(b, B - 1);
                box_grow(binBox[b], p.lo, p.hi);
                binCount[b]++;
            }
            float rightArea[64];
            uint32_t rightCount[64];
            Aabb acc;
            box_empty(acc);
            uint32_t cnt = 0;
            for (uint32_t b = B - 1; b > 0; --b) {
                box_grow(acc, binBox[b].lo, binBox[b].hi);
                cnt += binCount[b];
                rightArea[b] = box_area(acc);
                rightCount[b] = cnt;
            }
            box_empty(acc);
            cnt = 0;
            for (uint32_t b = 0; b + 1 < B; ++b) {
                box_grow(acc, binBox[b].lo, binBox[b].hi);
                cnt += binCount[b];
                if (cnt == 0 || rightCount[b + 1] == 0)
                    continue;
                const float cost = box_area(acc) * float(cnt) + rightArea[b + 1] * float(rightCount[b + 1]);
                if (cost < bestCost) {
                    bestCost = cost;
                    bestAxis = axis;
                    bestSplit = b + 1;
                }
            }
        }

        // leaf if allowed and cheaper (traversal step cost 1, intersection cost 1)
        const float leafCost = float(count);
        const float splitCost = parentArea > 0.f ? 1.f + bestCost / parentArea : INFINITY;
        if (count <= opt.maxLeafSize && (bestAxis < 0 || leafCost <= splitCost)) {
            make_leaf(nodeIx, begin, end, box);
            return;
        }

        uint32_t mid = begin;
        if (bestAxis >= 0) {
            const float extent = cbox.hi[bestAxis] - cbox.lo[bestAxis];
            const float k = float(B) / extent;
            const float lo = cbox.lo[bestAxis];
            uint32_t* it = std::partition(refs.data() + begin, refs.data() + end, [&](uint32_t r) {
                uint32_t b = uint32_t((prims[r].c[bestAxis] - lo) * k);
                b = std::min(b, B - 1);
                return b < bestSplit;
            });
            mid = uint32_t(it - refs.data());
        }
        if (mid == begin || mid == end) {
            // degenerate centroids: median split along the widest centroid axis
            int axis = 0;
            float ext = -1.f;
            for (int a = 0; a < 3; ++a) {
                const float e = cbox.hi[a] - cbox.lo[a];
                if (e > ext) {
                    ext = e;
                    axis = a;
                }
            }
            mid = begin + count / 2;
            std::nth_element(refs.data() + begin, refs.data() + mid, refs.data() + end,
                             [&](uint32_t x, uint32_t y) { return prims[x].c[axis] < prims[y].c[axis]; });
        }

        const uint32_t children = nodeCount.fetch_add(2);
        BinaryNode& n = nodes[nodeIx];
        n.box = box;
        n.left = children;
        n.count = 0;

        const bool spawn = count > 32768 && threadsLeft.fetch_sub(1) > 0;
        if (spawn) {
            std::thread t([this, children, begin, mid] { build(children, begin, mid); });
            build(children + 1, mid, end);
            t.join();
        } else {
            build(children, begin, mid);
            build(children + 1, mid, end);
        }
    }
};

inline uint8_t byte_of(const uint32_t* words, int i) { return uint8_t((words[i >> 2] >> ((i & 3) * 8)) & 0xff); }
inline void set_byte(uint32_t* words, int i, uint32_t v)
{
    words[i >> 2] &= ~(0xffu << ((i & 3) * 8));
    words[i >> 2] |= (v & 0xffu) << ((i & 3) * 8);
}

// A child of a wide node: binary subtree `bin`, either a leaf holding its
// `count` triangles (primRefs[first, first + count)) or an internal wide node.
struct Kid {
    uint32_t bin;
    bool leaf;
    uint32_t first;
    uint32_t count;
};

// SAH-optimal collapse of a binary BVH into 8-wide nodes (Ylitie, Karras, Laine,
// HPG 2017, section 3.1): for every binary node n and i = 1..8, the least SAH
// cost of representing n's subtree by at most i children of a wide node, where a
// child is a leaf of up to maxLeaf triangles (cost: area x kPrim per triangle) or
// an internal wide node (area x kNode, plus the cost of its own up-to-8 children).
struct SahCollapse {
    // tables written before they are read (children before parents), so left uninitialised
    std::unique_ptr<float[]> cost;       // 8 per binary node
    std::unique_ptr<uint8_t[]> choice;   // 8 per node: [0] 0 leaf / 1 internal; [i] 0xff like i-1, else slots k of the left child
    std::unique_ptr<uint8_t[]> split8;   // slots of the left child in the node's own 8 children
    std::unique_ptr<uint32_t[]> first, prims;
    const std::vector<BinaryNode>* bn = nullptr;
    uint32_t maxLeaf = 3;
    int spawnDepth = 0;

    SahCollapse() = default;
    SahCollapse(const BinaryBvh& bvh, uint32_t maxLeaf) : bn(&bvh.nodes), maxLeaf(maxLeaf)
    {
        const size_t n = bvh.nodes.size();
        cost.reset(new float[8 * n]);
        choice.reset(new uint8_t[8 * n]);
        split8.reset(new uint8_t[n]);
        first.reset(new uint32_t[n]);
        prims.reset(new uint32_t[n]);
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        while ((1u << spawnDepth) < hw)
            ++spawnDepth;
        solve(0, 0);
    }
    bool empty() const { return !cost; }

    // the table of node x after those of its subtree; the top levels split across threads
    void solve(uint32_t x, int depth)
    {
        const BinaryNode& b = (*bn)[x];
        if (b.count == 0) {
            const uint32_t l = b.left;
            if (depth < spawnDepth) {
                std::thread t([this, l, depth] { solve(l, depth + 1); });
                solve(l + 1, depth + 1);
                t.join();
            } else {
                solve(l, depth + 1);
                solve(l + 1, depth + 1);
            }
        }
        node(x);
    }

    void node(uint32_t x)
    {
        // a triangle test weighed as a node visit: with these kernels a node test (eight
        // slabs) and a triangle test (48 bytes) cost about alike, and this weight gave the
        // fewest node visits and triangle tests together on the benchmark heightfield
        constexpr float kNode = 1.f, kPrim = 1.f;
        const BinaryNode& b = (*bn)[x];
        const float area = box_area(b.box);
        float* c = &cost[8 * size_t(x)];
        uint8_t* ch = &choice[8 * size_t(x)];
        if (b.count > 0) {
            first[x] = b.left;
            prims[x] = b.count;
            const float leaf = b.count <= maxLeaf ? area * kPrim * float(b.count) : INFINITY;
            for (int i = 0; i < 8; ++i) {
                c[i] = leaf;
                ch[i] = i == 0 ? 0 : 0xff;
            }
            split8[x] = 0;
            return;
        }
        first[x] = first[b.left];
        prims[x] = prims[b.left] + prims[b.left + 1];
        const float leaf = prims[x] <= maxLeaf ? area * kPrim * float(prims[x]) : INFINITY;
        const float* cl = &cost[8 * size_t(b.left)];
        const float* cr = &cost[8 * size_t(b.left + 1)];
        float dist[9];
        uint8_t distK[9];
        for (int j = 2; j <= 8; ++j) {
            dist[j] = INFINITY;
            distK[j] = 1;
            for (int k = 1; k < j; ++k) {
                const float v = cl[k - 1] + cr[j - k - 1];
                if (v < dist[j]) {
                    dist[j] = v;
                    distK[j] = uint8_t(k);
                }
            }
        }
        split8[x] = distK[8];
        const float internal = area * kNode + dist[8];
        c[0] = leaf <= internal ? leaf : internal;
        ch[0] = leaf <= internal ? 0 : 1;
        for (int i = 1; i < 8; ++i) {
            if (dist[i + 1] < c[i - 1]) {
                c[i] = dist[i + 1];
                ch[i] = distK[i + 1];
            } else {
                c[i] = c[i - 1];
                ch[i] = 0xff;
            }
        }
    }

    // the children representing node x's subtree in at most i + 1 slots
    void gather(const std::vector<BinaryNode>& bn, uint32_t x, int i, Kid* out, int& count) const
    {
        while (i > 0 && choice[8 * size_t(x) + size_t(i)] == 0xff)
            --i;
        if (bn[x].count > 0) {
            out[count++] = Kid{x, true, bn[x].left, bn[x].count};
            return;
        }
        if (i == 0) {
            const bool leaf = choice[8 * size_t(x)] == 0;
            out[count++] = Kid{x, leaf, first[x], prims[x]};
            return;
        }
        const int k = choice[8 * size_t(x) + size_t(i)];
        gather(bn, bn[x].left, k - 1, out, count);
        gather(bn, bn[x].left + 1, i - k, out, count);
    }

    // the children of the wide node made for binary node x
    int children(const std::vector<BinaryNode>& bn, uint32_t x, Kid* out) const
    {
        int count = 0;
        if (bn[x].count > 0 || choice[8 * size_t(x)] == 0) {
            out[count++] = Kid{x, true, first[x], prims[x]};  // the whole subtree is one leaf
            return count;
        }
        const int k = split8[x];
        gather(bn, bn[x].left, k - 1, out, count);
        gather(bn, bn[x].left + 1, 8 - k - 1, out, count);
        return count;
    }
};

} // namespace

namespace {

BinaryBvh build_from_prims(const std::vector<PrimInfo>& prims, const BvhBuildOptions& options)
{
    BinaryBvh out;
    const uint32_t triCount = uint32_t(prims.size());
    out.primRefs.resize(triCount);
    for (uint32_t t = 0; t < triCount; ++t)
        out.primRefs[t] = t;
    out.nodes.resize(std::max<size_t>(1, 2 * size_t(triCount)));
    if (triCount == 0) {
        box_empty(out.nodes[0].box);
        out.nodes[0].left = 0;
        out.nodes[0].count = 0;
        out.nodes.resize(1);
        return out;
    }
    BvhBuildOptions opt = options;
    opt.maxLeafSize = std::max(1u, std::min(opt.maxLeafSize, 3u));
    BinaryBuilder b(prims, out.primRefs, out.nodes, opt);
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    b.threadsLeft = int(opt.threads ? opt.threads : hw) - 1;
    b.build(0, 0, triCount);
    out.nodes.resize(b.nodeCount.load());
    return out;
}

} // namespace

BinaryBvh build_binary_bvh(const float* positions, const uint32_t* indices, uint32_t triCount,
                           const BvhBuildOptions& options)
{
    std::vector<PrimInfo> prims(triCount);
    for (uint32_t t = 0; t < triCount; ++t) {
        PrimInfo& p = prims[t];
        for (int a = 0; a < 3; ++a) {
            const float x0 = positions[3 * indices[3 * t + 0] + a];
            const float x1 = positions[3 * indices[3 * t + 1] + a];
            const float x2 = positions[3 * indices[3 * t + 2] + a];
            p.lo[a] = std::min(x0, std::min(x1, x2));
            p.hi[a] = std::max(x0, std::max(x1, x2));
            p.c[a] = 0.5f * (p.lo[a] + p.hi[a]);
        }
    }
    return build_from_prims(prims, options);
}

Cwbvh build_cwbvh(const float* positions, const uint32_t* indices, uint32_t triCount, const BvhBuildOptions& opt,
                  Aabb* bounds)
{
    BvhBuildOptions o = opt;
    const uint32_t leaf = std::max(1u, std::min(opt.maxLeafSize, 3u));
    if (opt.sahCollapse)
        o.maxLeafSize = 1;
    const BinaryBvh bin = build_binary_bvh(positions, indices, triCount, o);
    if (bounds)
        *bounds = bin.nodes[0].box;
    return collapse_to_cwbvh(bin, positions, indices, opt.sahCollapse ? leaf : 0u);
}

BinaryBvh build_binary_bvh_boxes(const Aabb* boxes, uint32_t count, const BvhBuildOptions& options)
{
    std::vector<PrimInfo> prims(count);
    for (uint32_t i = 0; i < count; ++i)
        for (int a = 0; a < 3; ++a) {
            prims[i].lo[a] = boxes[i].lo[a];
            prims[i].hi[a] = boxes[i].hi[a];
            prims[i].c[a] = 0.5f * (boxes[i].lo[a] + boxes[i].hi[a]);
        }
    return build_from_prims(prims, options);
}

Cwbvh collapse_to_cwbvh(const BinaryBvh& bvh, const float* positions, const uint32_t* indices, uint32_t sahMaxLeaf)
{
    const SahCollapse sah = sahMaxLeaf && !bvh.primRefs.empty() ? SahCollapse(bvh, sahMaxLeaf) : SahCollapse();
    Cwbvh out;
    const std::vector<BinaryNode>& bn = bvh.nodes;
    out.nodes.push_back(WideNode{});
    if (bvh.primRefs.empty()) {
        // empty scene: a root without children never reports a hit
        return out;
    }

    // Layout pass (breadth first, sequential): the children of every wide node,
    // their slots, and where its internal children and leaf triangles go. Internal
    // children take consecutive wide indices in slot order, leaf triangles
    // consecutive slots in slot order.
    struct WideRec {
        uint32_t wide;
        uint32_t childBase;
        uint32_t triBase;
        int kidCount;
        Kid kids[8];
        int slotKid[8];
        Aabb box;
    };
    struct Task {
        uint32_t bin;
        uint32_t wide;
    };
    std::vector<WideRec> recs;
    recs.reserve(bn.size() / 4 + 1);
    std::deque<Task> tasks;
    tasks.push_back({0, 0});
    uint32_t nextWide = 1, nextTri = 0;
    const SahCollapse* dp = sah.empty() ? nullptr : &sah;
    while (!tasks.empty()) {
        const Task task = tasks.front();
        tasks.pop_front();
        WideRec rec;
        rec.wide = task.wide;

        // the up to 8 children of the wide node: binary subtrees, each a leaf
        // (its triangles tested together) or an internal wide node
        Kid* kids = rec.kids;
        int kidCount = 0;
        if (dp) {
            kidCount = dp->children(bn, task.bin, kids);
        } else {
            // greedy: repeatedly open the largest internal child
            uint32_t bins[8];
            if (bn[task.bin].count > 0) {
                bins[kidCount++] = task.bin;  // a leaf root
            } else {
                bins[kidCount++] = bn[task.bin].left;
                bins[kidCount++] = bn[task.bin].left + 1;
            }
            while (kidCount < 8) {
                int best = -1;
                float bestArea = -1.f;
                for (int k = 0; k < kidCount; ++k) {
                    if (bn[bins[k]].count == 0) {
                        const float a = box_area(bn[bins[k]].box);
                        if (a > bestArea) {
                            bestArea = a;
                            best = k;
                        }
                    }
                }
                if (best < 0)
                    break;
                const uint32_t opened = bins[best];
                bins[best] = bn[opened].left;
                bins[kidCount++] = bn[opened].left + 1;
            }
            for (int k = 0; k < kidCount; ++k)
                kids[k] = Kid{bins[k], bn[bins[k]].count > 0, bn[bins[k]].left, bn[bins[k]].count};
        }
        rec.kidCount = kidCount;

        Aabb& nodeBox = rec.box;
        box_empty(nodeBox);
        for (int k = 0; k < kidCount; ++k)
            box_grow(nodeBox, bn[kids[k].bin].box.lo, bn[kids[k].bin].box.hi);

        // slot assignment: slot s holds the child nearest for rays of octant s
        // (octant bit a set = negative direction along axis a)
        int* slotKid = rec.slotKid;
        for (int sl = 0; sl < 8; ++sl)
            slotKid[sl] = -1;
        {
            float cost[8][8];
            float pc[3];
            for (int a = 0; a < 3; ++a)
                pc[a] = 0.5f * (nodeBox.lo[a] + nodeBox.hi[a]);
            for (int k = 0; k < kidCount; ++k) {
                float c[3];
                for (int a = 0; a < 3; ++a)
                    c[a] = 0.5f * (bn[kids[k].bin].box.lo[a] + bn[kids[k].bin].box.hi[a]) - pc[a];
                for (int sl = 0; sl < 8; ++sl) {
                    const float dx = (sl & 1) ? -1.f : 1.f, dy = (sl & 2) ? -1.f : 1.f, dz = (sl & 4) ? -1.f : 1.f;
                    cost[k][sl] = c[0] * dx + c[1] * dy + c[2] * dz;
                }
            }
            bool kidDone[8] = {};
            for (int round = 0; round < kidCount; ++round) {
                float bc = INFINITY;
                int bk = -1, bs = -1;
                for (int k = 0; k < kidCount; ++k) {
                    if (kidDone[k])
                        continue;
                    for (int sl = 0; sl < 8; ++sl) {
                        if (slotKid[sl] >= 0)
                            continue;
                        if (cost[k][sl] < bc || bk < 0) {
                            bc = cost[k][sl];
                            bk = k;
                            bs = sl;
                        }
                    }
                }
                kidDone[bk] = true;
                slotKid[bs] = bk;
            }
        }

        rec.childBase = nextWide;
        rec.triBase = nextTri;
        for (int sl = 0; sl < 8; ++sl) {
            if (slotKid[sl] < 0)
                continue;
            const Kid& kk = kids[slotKid[sl]];
            if (!kk.leaf)
                tasks.push_back({kk.bin, nextWide++});
            else
                nextTri += kk.count;
        }
        recs.push_back(rec);
    }
    out.nodes.resize(nextWide);
    out.triPrim.resize(nextTri);
    if (positions)
        out.tris.resize(3 * size_t(nextTri));

    // Encoding pass (parallel over wide nodes): child boxes, meta bytes, the
    // node header and the traversal triangles of its leaves.
    auto encode = [&](const WideRec& rec) {
        WideNode node{};
        for (int a = 0; a < 3; ++a)
            for (int sl = 0; sl < 8; ++sl) {
                node.lo[a][sl] = INFINITY;
                node.hi[a][sl] = -INFINITY;
            }
        uint32_t meta[2] = {0, 0};
        uint32_t triCount = 0;
        for (int sl = 0; sl < 8; ++sl) {
            if (rec.slotKid[sl] < 0)
                continue;
            const Kid& kk = rec.kids[rec.slotKid[sl]];
            const BinaryNode& kid = bn[kk.bin];
            for (int a = 0; a < 3; ++a) {
                node.lo[a][sl] = kid.box.lo[a];
                node.hi[a][sl] = kid.box.hi[a];
            }
            if (!kk.leaf) {
                set_byte(meta, sl, 0x20u | (24u + uint32_t(sl)));
            } else {
                const uint32_t unary = (1u << kk.count) - 1u;
                set_byte(meta, sl, (unary << 5) | triCount);
                for (uint32_t i = 0; i < kk.count; ++i) {
                    const uint32_t prim = bvh.primRefs[kk.first + i];
                    const size_t slot = size_t(rec.triBase) + triCount + i;
                    out.triPrim[slot] = prim;
                    if (!positions)  // a BVH over boxes: the leaf slot only names the primitive
                        continue;
                    const float* p0 = positions + 3 * indices[3 * prim + 0];
                    const float* p1 = positions + 3 * indices[3 * prim + 1];
                    const float* p2 = positions + 3 * indices[3 * prim + 2];
                    out.tris[3 * slot + 0] = make_float4(p0[0], p0[1], p0[2], u2f(prim));
                    out.tris[3 * slot + 1] = make_float4(p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], 0.f);
                    out.tris[3 * slot + 2] = make_float4(p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2], 0.f);
                }
                triCount += kk.count;
            }
        }
        node.hdr = make_uint4(rec.childBase, rec.triBase, meta[0], meta[1]);
        out.nodes[rec.wide] = node;
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned workers = recs.size() > 4096 ? hw : 1u;
    std::atomic<size_t> next{0};
    auto run = [&] {
        constexpr size_t kChunk = 256;
        for (size_t b0 = next.fetch_add(kChunk); b0 < recs.size(); b0 = next.fetch_add(kChunk))
            for (size_t i = b0; i < std::min(recs.size(), b0 + kChunk); ++i)
                encode(recs[i]);
    };
    std::vector<std::thread> pool;
    for (unsigned w = 1; w < workers; ++w)
        pool.emplace_back(run);
    run();
    for (std::thread& t : pool)
        t.join();
    return out;
}
std::vector<QuantNode> quantize_nodes(const std::vector<WideNode>& nodes)
{
    std::vector<QuantNode> out(nodes.size());
    for (size_t n = 0; n < nodes.size(); ++n) {
        const WideNode& w = nodes[n];
        const uint32_t meta[2] = {w.hdr.z, w.hdr.w};
        auto metaOf = [&](int sl) { return (meta[sl >> 2] >> (8 * (sl & 3))) & 0xffu; };
        Aabb box;
        for (int a = 0; a < 3; ++a) {
            box.lo[a] = INFINITY;
            box.hi[a] = -INFINITY;
        }
        for (int sl = 0; sl < 8; ++sl)
            if (metaOf(sl))
                for (int a = 0; a < 3; ++a) {
                    box.lo[a] = std::min(box.lo[a], w.lo[a][sl]);
                    box.hi[a] = std::max(box.hi[a], w.hi[a][sl]);
                }
        uint32_t w0[4] = {0, 0, 0, 0};
        uint32_t q[6][2] = {};  // qlo.x, qlo.y, qlo.z, qhi.x, qhi.y, qhi.z
        double scale[3];
        for (int a = 0; a < 3; ++a) {
            if (!(box.lo[a] <= box.hi[a]))
                box.lo[a] = box.hi[a] = 0.f;  // no child
            const double extent = double(box.hi[a]) - double(box.lo[a]);
            int e = -100;
            if (extent > 0.0) {
                int ex;
                std::frexp(extent / 255.0, &ex);
                e = ex;
            }
            e = std::max(-126, std::min(e, 127));
            scale[a] = std::ldexp(1.0, e);
            w0[a] = f2u(box.lo[a]);
            w0[3] |= uint32_t(e + 127) << (8 * a);
        }
        uint32_t imask = 0;
        for (int sl = 0; sl < 8; ++sl) {
            const uint32_t m = metaOf(sl);
            if (!m)
                continue;
            if ((m & 0x1fu) >= 24u)
                imask |= 1u << sl;
            for (int a = 0; a < 3; ++a) {
                const double lo = (double(w.lo[a][sl]) - double(box.lo[a])) / scale[a];
                const double hi = (double(w.hi[a][sl]) - double(box.lo[a])) / scale[a];
                set_byte(q[a], sl, uint32_t(std::max(0, std::min(255, int(std::floor(lo))))));
                set_byte(q[3 + a], sl, uint32_t(std::max(0, std::min(255, int(std::ceil(hi))))));
            }
        }
        w0[3] |= imask << 24;
        QuantNode& o = out[n];
        o.w[0] = make_uint4(w0[0], w0[1], w0[2], w0[3]);
        o.w[1] = w.hdr;
        o.w[2] = make_uint4(q[0][0], q[0][1], q[1][0], q[1][1]);
        o.w[3] = make_uint4(q[2][0], q[2][1], q[3][0], q[3][1]);
        o.w[4] = make_uint4(q[4][0], q[4][1], q[5][0], q[5][1]);
    }
    return out;
}

} // namespace tr
