// Batched rendering: many independent scenes of uneven triangle count,
// resolution and sample count rendered by one continuous wavefront. No
// counterpart in the reference, whose DeviceRenderer renders one scene at a
// time with a host bounce loop (Tracer/Renderer/DeviceRenderer.cpp:97-133,
// with a blocking counter download per bounce at :255-257).
//
// Every item's scene is flattened and given its own 8-wide BVH (built on host
// threads, one item per thread); the buffers are concatenated into one device
// arena with node, triangle, material and light indices rebased, so a ray
// only needs its item's root node. All items' samples are numbered (a sample
// id: item by item, pixel by pixel, the samples of a pixel consecutive) and
// fed to a pool of path slots from a device cursor: each iteration traces the
// paths the last one carried over plus new samples in the slots that ended
// paths left, so the pool stays full until the last samples drain, with no
// per-scene or per-wave tail. The iterations run as a CUDA graph while loop
// whose condition a device plan kernel sets (queue not empty), so one
// tr_batch_render is one graph launch with no host round trip. Each sample's
// radiance lands in a per-sample buffer, summed per pixel in sample order at
// the end; items whose samples exceed that buffer's budget go to the next
// round (the rounds run one after the other in the same graph).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/trayracer.h"
#include "tr_api_internal.h"
#include "tr_bvh.h"
#include "tr_continuous.h"
#include "tr_kernels.h"
#include "tr_scene.h"

namespace {

using namespace tr;

constexpr uint64_t kDefaultPoolPaths = 1ull << 25;
// Samples of one round: the per-sample radiance buffer holds this many float4.
constexpr uint64_t kRoundSamples = 1ull << 30;

// Consecutive items whose samples share one per-sample radiance buffer.
struct Round {
    uint32_t firstItem = 0;
    uint32_t itemCount = 0;
    uint32_t samples = 0;     // sample ids [0, samples) of the round
    uint32_t pixelBegin = 0;  // the round's pixels in the batch accumulator
    uint32_t pixelEnd = 0;
};

struct ItemBuild {
    FlatScene flat;
    Cwbvh bvh;
    uint32_t triangles = 0;
    std::string error;
};

struct Batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    // a captured iteration traces the last iteration's shadow rays on `side`
    // while its extend runs on `stream` (fork / join)
    cudaStream_t side = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    std::string lastError;

    void* sceneArena = nullptr;
    std::vector<cudaArray_t> texArrays;            // the items' textures
    std::vector<cudaTextureObject_t> texObjects;
    void* frameArena = nullptr;
    SceneView scene{};
    FrameView frame{};               // pool buffers; items, item count and state set per round
    std::vector<Round> rounds;
    std::vector<BatchItem> items;
    BatchItem* itemsDevice = nullptr;
    BatchState* states = nullptr;    // one per round
    float4* accumulator = nullptr;
    float4* colors = nullptr;
    uint32_t pool = 0;               // path slots
    LaunchShape shape{};
    tr_batch_info info{};

    Settings graphSettings{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    bool graphValid = false;
    cudaEvent_t evStart = nullptr, evStop = nullptr;
    Settings lastSettings{};
    bool rendered = false;
};

tr_status fail(Batch* b, tr_status st, const std::string& msg)
{
    if (b)
        b->lastError = msg;
    return st;
}

tr_status cuda_fail(Batch* b, cudaError_t e, const char* what)
{
    const bool sticky = e == cudaErrorIllegalAddress || e == cudaErrorLaunchFailure ||
                        e == cudaErrorIllegalInstruction || e == cudaErrorMisalignedAddress ||
                        e == cudaErrorHardwareStackError || e == cudaErrorAssert;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(b, TR_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
    }
    return fail(b, sticky ? TR_ERR_DEVICE_FAULT : TR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define TR_BCUDA(b, call)                                   \
    do {                                                    \
        const cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess)                              \
            return cuda_fail((b), e_, #call);               \
    } while (0)

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

void release_graph(Batch* b)
{
    if (b->graphExec)
        cudaGraphExecDestroy(b->graphExec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    b->graphExec = nullptr;
    b->graph = nullptr;
    b->graphValid = false;
}

void release(Batch* b)
{
    release_graph(b);
    if (b->evStart)
        cudaEventDestroy(b->evStart);
    if (b->evStop)
        cudaEventDestroy(b->evStop);
    if (b->sceneArena)
        cudaFree(b->sceneArena);
    for (cudaTextureObject_t t : b->texObjects)
        cudaDestroyTextureObject(t);
    for (cudaArray_t a : b->texArrays)
        cudaFreeArray(a);
    if (b->frameArena)
        cudaFree(b->frameArena);
    if (b->evFork)
        cudaEventDestroy(b->evFork);
    if (b->evJoin)
        cudaEventDestroy(b->evJoin);
    if (b->side)
        cudaStreamDestroy(b->side);
    if (b->stream)
        cudaStreamDestroy(b->stream);
}

// Flattens and builds the BVH of every item, one item per host thread.
std::vector<ItemBuild> build_items(const tr_batch_item* items, uint32_t count, uint32_t leafSize)
{
    std::vector<ItemBuild> out(count);
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        for (uint32_t i = next++; i < count; i = next++) {
            const tr_scene_desc& d = *items[i].scene;
            ItemBuild& r = out[i];
            try {
                r.flat = flatten_scene(d);
                BvhBuildOptions opt;
                opt.maxLeafSize = d.bvh_leaf_size ? d.bvh_leaf_size : leafSize;
                opt.threads = 1;
                const tr_mesh_desc& m = *d.mesh;
                r.bvh = build_cwbvh(m.positions, m.indices, m.triangle_count, opt);
                r.triangles = m.triangle_count;
            } catch (const std::exception& e) {
                r.error = e.what();
            }
        }
    };
    const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
    const uint32_t n = std::min(count, hw);
    std::vector<std::thread> pool;
    for (uint32_t t = 1; t < n; ++t)
        pool.emplace_back(worker);
    worker();
    for (auto& t : pool)
        t.join();
    return out;
}

// Items in order into rounds of at most kRoundSamples samples; sample ids
// (BatchItem::sampleBase) count from each round's first item.
bool plan_rounds(std::vector<BatchItem>& items, std::vector<Round>& rounds)
{
    Round r{};
    uint64_t samples = 0;
    for (uint32_t i = 0; i < items.size(); ++i) {
        const uint64_t n = uint64_t(items[i].width) * items[i].height * items[i].spp;
        if (n > kRoundSamples)
            return false;
        if (samples + n > kRoundSamples) {
            r.samples = uint32_t(samples);
            rounds.push_back(r);
            r = Round{};
            r.firstItem = i;
            r.pixelBegin = items[i].pixelBase;
            samples = 0;
        }
        items[i].sampleBase = uint32_t(samples);
        samples += n;
        r.itemCount++;
        r.pixelEnd = items[i].pixelBase + items[i].width * items[i].height;
    }
    if (r.itemCount) {
        r.samples = uint32_t(samples);
        rounds.push_back(r);
    }
    return true;
}

FrameView round_view(const Batch* b, uint32_t k)
{
    FrameView f = b->frame;
    const Round& r = b->rounds[k];
    f.items = b->itemsDevice + r.firstItem;
    f.itemCount = r.itemCount;
    f.batch = b->states + k;
    return f;
}

// The rounds as the continuous wavefront runs them.
std::vector<ContinuousRound> continuous_rounds(const Batch* b)
{
    std::vector<ContinuousRound> out;
    for (uint32_t k = 0; k < b->rounds.size(); ++k) {
        const Round& r = b->rounds[k];
        out.push_back(ContinuousRound{round_view(b, k), r.samples, r.pixelBegin, r.pixelEnd});
    }
    return out;
}

ContinuousLaunch continuous_launch(const Batch* b, const Settings& st)
{
    return ContinuousLaunch{b->scene, st, b->shape, b->pool, b->side, b->evFork, b->evJoin};
}

} // namespace

extern "C" {

tr_status tr_batch_create(const tr_config* config, const tr_batch_item* items, uint32_t count,
                          uint64_t pool_paths, void** out_batch)
{
    if (!config || !out_batch || !items || count == 0)
        return TR_ERR_INVALID_ARGUMENT;
    *out_batch = nullptr;
    if (config->abi_version != TR_ABI_VERSION)
        return TR_ERR_INVALID_ARGUMENT;
    const uint64_t poolCap = pool_paths ? pool_paths : kDefaultPoolPaths;
    if (poolCap >= TR_MAX_PATHS || count >= (1u << 24))  // a path keeps its item in 24 bits
        return TR_ERR_LIMIT;
    uint64_t pixels = 0, paths = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const tr_batch_item& it = items[i];
        if (!it.scene || it.width == 0 || it.height == 0 || it.spp == 0)
            return TR_ERR_INVALID_ARGUMENT;
        if (uint64_t(it.width) * it.height * it.spp > kRoundSamples)
            return TR_ERR_LIMIT;
        if (!validate_scene(*it.scene).empty() || it.scene->instance_count)
            return TR_ERR_INVALID_ARGUMENT;  // one-mesh scenes only
        pixels += uint64_t(it.width) * it.height;
        paths += uint64_t(it.width) * it.height * it.spp;
    }
    if (pixels >= (1ull << 32))
        return TR_ERR_LIMIT;
    if (cudaSetDevice(config->device) != cudaSuccess)
        return TR_ERR_CUDA;

    Batch* b = new (std::nothrow) Batch();
    if (!b)
        return TR_ERR_OUT_OF_MEMORY;
    b->device = config->device;
    auto bail = [&](tr_status st) {
        release(b);
        delete b;
        return st;
    };
    // a blocking stream, like the context's: work on it is ordered with the legacy default stream
    if (cudaStreamCreate(&b->stream) != cudaSuccess || cudaEventCreate(&b->evStart) != cudaSuccess ||
        cudaEventCreate(&b->evStop) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->evFork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->evJoin, cudaEventDisableTiming) != cudaSuccess)
        return bail(TR_ERR_CUDA);

    const auto t0 = std::chrono::steady_clock::now();
    std::vector<ItemBuild> built = build_items(items, count, 3u);
    for (const ItemBuild& r : built)
        if (!r.error.empty())
            return bail(TR_ERR_INVALID_ARGUMENT);

    // concatenated host buffers with rebased indices
    std::vector<WideNode> nodes;
    std::vector<float4> btris;
    std::vector<TriShade> tris;
    std::vector<uint32_t> matIdx;
    std::vector<Material> materials;
    std::vector<LightTri> lights;
    std::vector<AliasEntry> alias;
    std::vector<TexSlots> texSlots;  // per material, when an item has textures
    bool anyTextures = false;
    for (uint32_t i = 0; i < count; ++i)
        anyTextures |= !built[i].flat.texSlots.empty();
    b->items.resize(count);
    uint64_t pixelBase = 0, triTotal = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const ItemBuild& r = built[i];
        const uint32_t nodeBase = uint32_t(nodes.size());
        const uint32_t slotBase = uint32_t(btris.size() / 3);
        const uint32_t primBase = uint32_t(tris.size());
        const uint32_t matBase = uint32_t(materials.size());
        const uint32_t lightBase = uint32_t(lights.size());
        for (WideNode n : r.bvh.nodes) {
            n.hdr.x += nodeBase;
            n.hdr.y += slotBase;
            nodes.push_back(n);
        }
        for (size_t k = 0; k < r.bvh.tris.size(); ++k) {
            float4 v = r.bvh.tris[k];
            if (k % 3 == 0) {
                uint32_t prim;
                std::memcpy(&prim, &v.w, 4);
                prim += primBase;
                std::memcpy(&v.w, &prim, 4);
            }
            btris.push_back(v);
        }
        tris.insert(tris.end(), r.flat.tris.begin(), r.flat.tris.end());
        for (uint32_t m : r.flat.matIdx)
            matIdx.push_back(m + matBase);
        materials.insert(materials.end(), r.flat.materials.begin(), r.flat.materials.end());
        if (anyTextures) {
            // the item's textures as texture objects; its slots name them (index + 1 before)
            const size_t texBase = b->texObjects.size();
            const tr_scene_desc& sd = *items[i].scene;
            for (uint32_t k = 0; !r.flat.texSlots.empty() && k < sd.texture_count; ++k) {
                cudaArray_t arr = nullptr;
                cudaTextureObject_t obj = 0;
                const cudaError_t te = create_texture(sd.textures[k], &arr, &obj);
                if (arr)
                    b->texArrays.push_back(arr);
                if (te != cudaSuccess) {
                    cudaGetLastError();
                    return bail(te == cudaErrorMemoryAllocation ? TR_ERR_OUT_OF_MEMORY : TR_ERR_CUDA);
                }
                b->texObjects.push_back(obj);
            }
            if (r.flat.texSlots.empty()) {
                texSlots.resize(texSlots.size() + r.flat.materials.size(), TexSlots{});
            } else {
                for (TexSlots slot : r.flat.texSlots) {
                    for (uint32_t p = 0; p < TR_PROP_COUNT; ++p)
                        if (slot.tex[p])
                            slot.tex[p] = b->texObjects[texBase + size_t(slot.tex[p] - 1u)];
                    texSlots.push_back(slot);
                }
            }
        }
        for (LightTri L : r.flat.lights) {
            L.triIx += int32_t(primBase);
            lights.push_back(L);
        }
        alias.insert(alias.end(), r.flat.alias.begin(), r.flat.alias.end());

        BatchItem& it = b->items[i];
        it = BatchItem{};
        std::string err;
        if (!convert_camera(items[i].camera, &it.camera, &err))
            return bail(TR_ERR_INVALID_ARGUMENT);
        it.width = items[i].width;
        it.height = items[i].height;
        it.root = nodeBase;
        it.lightBase = lightBase;
        it.lightCount = int32_t(r.flat.lights.size());
        it.lightEnergy = r.flat.lightEnergy;
        it.lightEnergyTotal = r.flat.lightEnergyTotal;
        it.pixelBase = uint32_t(pixelBase);
        it.spp = items[i].spp;
        pixelBase += uint64_t(it.width) * it.height;
        triTotal += r.triangles;
    }
    built.clear();
    const float4 identity[3] = {make_float4(1.f, 0.f, 0.f, 0.f), make_float4(0.f, 1.f, 0.f, 0.f),
                                make_float4(0.f, 0.f, 1.f, 0.f)};
    if (!plan_rounds(b->items, b->rounds))
        return bail(TR_ERR_LIMIT);
    uint32_t roundSamples = 0;
    for (const Round& r : b->rounds)
        roundSamples = std::max(roundSamples, r.samples);
    const auto t1 = std::chrono::steady_clock::now();

    // scene arena
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + std::max<size_t>(bytes, 16));
        return o;
    };
    // the node layout of the concatenated BVHs (fp32 child boxes while they fit L2)
    const bool quant = quantized_nodes(nodes.size(), 0u);
    const std::vector<QuantNode> qnodes = quant ? quantize_nodes(nodes) : std::vector<QuantNode>{};
    const void* nodeSrc = quant ? static_cast<const void*>(qnodes.data()) : static_cast<const void*>(nodes.data());
    const size_t nodeBytes = nodes.size() * (quant ? sizeof(QuantNode) : sizeof(WideNode));
    const size_t oNodes = take(nodeBytes);
    const size_t oBTris = take(btris.size() * sizeof(float4));
    const size_t oTris = take(tris.size() * sizeof(TriShade));
    const size_t oMat = take(matIdx.size() * sizeof(uint32_t));
    const size_t oMats = take(materials.size() * sizeof(Material));
    const size_t oLights = take(lights.size() * sizeof(LightTri));
    const size_t oAlias = take(alias.size() * sizeof(AliasEntry));
    const size_t oXf = take(sizeof(identity));
    const size_t oTex = take(texSlots.size() * sizeof(TexSlots));
    const size_t sceneBytes = off;
    cudaError_t e = cudaMalloc(&b->sceneArena, sceneBytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bail(e == cudaErrorMemoryAllocation ? TR_ERR_OUT_OF_MEMORY : TR_ERR_CUDA);
    }
    char* sb = static_cast<char*>(b->sceneArena);
    auto up = [&](size_t o, const void* src, size_t bytes) {
        return bytes ? cudaMemcpy(sb + o, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
    };
    const cudaError_t es[] = {
        up(oNodes, nodeSrc, nodeBytes),
        up(oBTris, btris.data(), btris.size() * sizeof(float4)),
        up(oTris, tris.data(), tris.size() * sizeof(TriShade)),
        up(oMat, matIdx.data(), matIdx.size() * sizeof(uint32_t)),
        up(oMats, materials.data(), materials.size() * sizeof(Material)),
        up(oLights, lights.data(), lights.size() * sizeof(LightTri)),
        up(oAlias, alias.data(), alias.size() * sizeof(AliasEntry)),
        up(oXf, identity, sizeof(identity)),
        up(oTex, texSlots.data(), texSlots.size() * sizeof(TexSlots)),
    };
    for (cudaError_t x : es)
        if (x != cudaSuccess)
            return bail(TR_ERR_CUDA);
    SceneView& sv = b->scene;
    sv.nodes = sb + oNodes;
    sv.quantNodes = quant ? 1u : 0u;
    sv.bvhTris = reinterpret_cast<const float4*>(sb + oBTris);
    sv.tris = reinterpret_cast<const TriShade*>(sb + oTris);
    sv.matIdx = reinterpret_cast<const uint32_t*>(sb + oMat);
    sv.materials = reinterpret_cast<const Material*>(sb + oMats);
    sv.lights = reinterpret_cast<const LightTri*>(sb + oLights);
    sv.alias = reinterpret_cast<const AliasEntry*>(sb + oAlias);
    sv.invTransforms = reinterpret_cast<const float4*>(sb + oXf);
    sv.texSlots = texSlots.empty() ? nullptr : reinterpret_cast<const TexSlots*>(sb + oTex);
    sv.nodeCount = uint32_t(nodes.size());
    sv.triCount = uint32_t(tris.size());

    // frame arena: the pool's queues, the per-sample radiance of a round, the
    // batch accumulator and colors, items and round states
    const uint32_t pool = uint32_t(std::min<uint64_t>(poolCap, std::max<uint64_t>(1, roundSamples)));
    const size_t capN = pool;
    off = 0;
    const size_t oS0 = take(3 * capN * sizeof(float4));
    const size_t oS1 = take(3 * capN * sizeof(float4));
    const size_t oHits = take(capN * sizeof(uint4));
    const size_t oShadow = take(3 * capN * sizeof(float4));
    const size_t oRad = take(size_t(roundSamples) * sizeof(float4));
    const size_t oAcc = take(pixels * sizeof(float4));
    const size_t oCol = take(pixels * sizeof(float4));
    const size_t oItems = take(b->items.size() * sizeof(BatchItem));
    const size_t oStates = take(b->rounds.size() * sizeof(BatchState));
    const size_t oWords = take(2 * sizeof(uint32_t));
    const size_t oTrav = take(kTraversalCounters * sizeof(unsigned long long));
    e = cudaMalloc(&b->frameArena, off);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bail(e == cudaErrorMemoryAllocation ? TR_ERR_OUT_OF_MEMORY : TR_ERR_CUDA);
    }
    char* fb = static_cast<char*>(b->frameArena);
    if (cudaMemset(fb + oAcc, 0, oItems - oAcc) != cudaSuccess ||
        cudaMemset(fb + oStates, 0, off - oStates) != cudaSuccess ||
        cudaMemcpy(fb + oItems, b->items.data(), b->items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice) !=
            cudaSuccess)
        return bail(TR_ERR_CUDA);
    FrameView& f = b->frame;
    f = FrameView{};
    f.state[0] = reinterpret_cast<float4*>(fb + oS0);
    f.state[1] = reinterpret_cast<float4*>(fb + oS1);
    f.hits = reinterpret_cast<uint4*>(fb + oHits);
    f.shadow = reinterpret_cast<float4*>(fb + oShadow);
    f.radiance = reinterpret_cast<float4*>(fb + oRad);
    f.accumulator = reinterpret_cast<float4*>(fb + oAcc);
    f.colors = reinterpret_cast<float4*>(fb + oCol);
    f.albedo = nullptr;
    f.normals = nullptr;
    f.sampleCount = reinterpret_cast<uint32_t*>(fb + oWords);  // stays 0: samples are keyed per item
    f.errorFlag = reinterpret_cast<uint32_t*>(fb + oWords) + 1;
    f.traversal = reinterpret_cast<unsigned long long*>(fb + oTrav);
    f.capacity = pool;
    f.resX = 1;
    f.resY = 1;
    f.pathCount = pool;
    b->itemsDevice = reinterpret_cast<BatchItem*>(fb + oItems);
    b->states = reinterpret_cast<BatchState*>(fb + oStates);
    b->accumulator = f.accumulator;
    b->colors = f.colors;
    b->pool = pool;
    b->shape = default_launch_shape(b->device, pool);
    const auto t2 = std::chrono::steady_clock::now();

    tr_batch_info& in = b->info;
    in.item_count = count;
    in.round_count = uint32_t(b->rounds.size());
    in.path_count = paths;
    in.pixel_count = pixels;
    in.triangle_count = triTotal;
    in.device_bytes = sceneBytes + off;
    in.pool_paths = pool;
    in.build_time_ms = std::chrono::duration<float, std::milli>(t1 - t0).count();
    in.upload_time_ms = std::chrono::duration<float, std::milli>(t2 - t1).count();
    *out_batch = b;
    return TR_OK;
}

tr_status tr_batch_destroy(void* batch)
{
    if (!batch)
        return TR_ERR_INVALID_ARGUMENT;
    Batch* b = static_cast<Batch*>(batch);
    cudaSetDevice(b->device);
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    release(b);
    delete b;
    return TR_OK;
}

const char* tr_batch_last_error(void* batch)
{
    return batch ? static_cast<Batch*>(batch)->lastError.c_str() : "null batch";
}

tr_status tr_batch_get_info(void* batch, tr_batch_info* out)
{
    if (!batch || !out)
        return TR_ERR_INVALID_ARGUMENT;
    *out = static_cast<Batch*>(batch)->info;
    return TR_OK;
}

} // extern "C"

extern "C" {

tr_status tr_batch_render(void* batch, void* stream, const tr_kernel_settings* settings, int32_t use_graph)
{
    if (!batch || !settings)
        return TR_ERR_INVALID_ARGUMENT;
    Batch* b = static_cast<Batch*>(batch);
    Settings st{};
    std::string err;
    if (!convert_settings(*settings, &st, &err))
        return fail(b, TR_ERR_INVALID_ARGUMENT, err);
    if (st.flags & (TR_FLAG_REFERENCE_SAMPLING | TR_FLAG_WRITE_AOVS | TR_FLAG_REFERENCE_DRAW_RTL))
        return fail(b, TR_ERR_INVALID_ARGUMENT,
                    "batched rendering uses the default sampling mode and writes no guide buffers");
    st.multiSample = 1;  // unused: each item renders its own spp
    cudaSetDevice(b->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->stream;
    if (use_graph && !(st.flags & TR_FLAG_COUNT_TRAVERSAL) &&
        (!b->graphValid || std::memcmp(&st, &b->graphSettings, sizeof(Settings)) != 0)) {
        // captured on the batch's own stream, which must be idle
        TR_BCUDA(b, cudaStreamSynchronize(b->stream));
        release_graph(b);
        cudaGraph_t g = nullptr;
        TR_BCUDA(b, capture_continuous(continuous_launch(b, st), continuous_rounds(b), 0u, b->stream, &g));
        b->graph = g;
        TR_BCUDA(b, cudaGraphInstantiate(&b->graphExec, g, 0));
        b->graphValid = true;
        b->graphSettings = st;
    }
    TR_BCUDA(b, cudaEventRecord(b->evStart, s));
    TR_BCUDA(b, cudaMemsetAsync(b->frame.errorFlag, 0, sizeof(uint32_t), s));
    if (use_graph && !(st.flags & TR_FLAG_COUNT_TRAVERSAL)) {
        TR_BCUDA(b, cudaGraphLaunch(b->graphExec, s));
    } else {
        if (st.flags & TR_FLAG_COUNT_TRAVERSAL)
            TR_BCUDA(b, cudaMemsetAsync(b->frame.traversal, 0, kTraversalCounters * sizeof(unsigned long long), s));
        TR_BCUDA(b, run_continuous_eager(continuous_launch(b, st), continuous_rounds(b), 0u, s));
    }
    TR_BCUDA(b, cudaEventRecord(b->evStop, s));
    b->lastSettings = st;
    b->rendered = true;
    return TR_OK;
}

tr_status tr_batch_get_statistics(void* batch, tr_batch_statistics* out)
{
    if (!batch || !out)
        return TR_ERR_INVALID_ARGUMENT;
    Batch* b = static_cast<Batch*>(batch);
    if (!b->rendered)
        return fail(b, TR_ERR_NOT_READY, "no batch rendered");
    cudaSetDevice(b->device);
    TR_BCUDA(b, cudaEventSynchronize(b->evStop));
    std::vector<BatchState> states(b->rounds.size());
    TR_BCUDA(b, cudaMemcpy(states.data(), b->states, states.size() * sizeof(BatchState), cudaMemcpyDeviceToHost));
    uint32_t err = 0;
    unsigned long long trav[kTraversalCounters] = {};
    TR_BCUDA(b, cudaMemcpy(&err, b->frame.errorFlag, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    TR_BCUDA(b, cudaMemcpy(trav, b->frame.traversal, sizeof(trav), cudaMemcpyDeviceToHost));
    tr_batch_statistics s{};
    for (const BatchState& bs : states) {
        // the last plan of a round added its final iteration's counts
        s.extend_rays += bs.extendRays;
        s.shadow_rays += bs.shadowRays;
        s.hit_rays += bs.hitRays;
        s.iterations += bs.iterations;
    }
    // per round: start, finalize, and plan + extend + shade + connect per iteration (the last
    // iteration of a round finds nothing to trace)
    // kernels: per round its finalize and plan + connect + extend + shade per iteration (the
    // last finds nothing to trace); the round-start memset is not a kernel
    s.launches = uint32_t(b->rounds.size()) + 4u * (s.iterations + uint32_t(b->rounds.size()));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->evStart, b->evStop);
    s.render_time_ms = ms;
    s.device_error = err;
    s.traversal_extend_nodes = trav[0];
    s.traversal_extend_tris = trav[1];
    s.traversal_connect_nodes = trav[2];
    s.traversal_connect_tris = trav[3];
    *out = s;
    return TR_OK;
}

tr_status tr_batch_get_colors(void* batch, uint32_t item, void** device_rgba)
{
    if (!batch || !device_rgba)
        return TR_ERR_INVALID_ARGUMENT;
    Batch* b = static_cast<Batch*>(batch);
    if (item >= b->items.size())
        return fail(b, TR_ERR_INVALID_ARGUMENT, "item index out of range");
    *device_rgba = b->colors + b->items[item].pixelBase;
    return TR_OK;
}

tr_status tr_batch_download(void* batch, void* stream, uint32_t item, float* host_rgba, uint64_t bytes)
{
    if (!batch || !host_rgba)
        return TR_ERR_INVALID_ARGUMENT;
    Batch* b = static_cast<Batch*>(batch);
    if (item >= b->items.size())
        return fail(b, TR_ERR_INVALID_ARGUMENT, "item index out of range");
    const BatchItem& it = b->items[item];
    const uint64_t need = uint64_t(it.width) * it.height * sizeof(float4);
    if (bytes < need)
        return fail(b, TR_ERR_INVALID_ARGUMENT, "host buffer smaller than width * height * 16 bytes");
    if (!b->rendered)
        return fail(b, TR_ERR_NOT_READY, "no batch rendered");
    cudaSetDevice(b->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : b->stream;
    TR_BCUDA(b, cudaEventSynchronize(b->evStop));  // the render may have run on another stream
    TR_BCUDA(b, cudaMemcpyAsync(host_rgba, b->colors + it.pixelBase, need, cudaMemcpyDeviceToHost, s));
    TR_BCUDA(b, cudaStreamSynchronize(s));
    return TR_OK;
}

} // extern "C"
