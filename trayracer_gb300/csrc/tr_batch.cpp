// Batched rendering: many independent scenes of uneven triangle count,
// resolution and sample count rendered by one wavefront. No counterpart in
// the reference, whose DeviceRenderer renders one scene at a time
// (Tracer/Renderer/DeviceRenderer.cpp:97-133).
//
// Every item's scene is flattened and given its own 8-wide BVH (built on host
// threads, one item per thread); the buffers are concatenated into one device
// arena with node, triangle, material and light indices rebased, so a ray
// only needs its item's root node. The items' paths are cut into waves of at
// most `wave_paths` paths made of consecutive (item, sample) units; each wave
// runs the same generate / extend / shade / connect launches as one scene,
// with the item of a path looked up from the wave's segment table, and adds
// its samples to the batch accumulator. Two waves are in flight at a time, on
// two streams with their own buffers, so one wave's short late bounces overlap
// the other wave's long early ones; only the waves' accumulator updates are
// ordered. One tr_batch_render replays all waves from one CUDA graph.
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
#include "tr_kernels.h"
#include "tr_scene.h"

namespace {

using namespace tr;

constexpr uint64_t kDefaultWavePaths = 1ull << 25;
constexpr uint32_t kWaveSets = 2;  // waves in flight, each with its own buffers and stream

struct Wave {
    uint32_t segmentOffset = 0;
    uint32_t segmentCount = 0;
    uint32_t paths = 0;
    uint32_t pixels = 0;
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
    std::string lastError;

    void* sceneArena = nullptr;
    void* frameArena = nullptr;
    SceneView scene{};
    FrameView frame[kWaveSets]{};    // wave buffers of each set; segments, counts and counters set per wave
    cudaStream_t lanes[kWaveSets] = {};
    cudaEvent_t evFork = nullptr;
    std::vector<cudaEvent_t> evFinal; // per wave: its samples are in the accumulator
    std::vector<Wave> waves;
    std::vector<BatchItem> items;
    BatchSegment* segments = nullptr;
    uint32_t* counters = nullptr;    // kCounterWords per wave
    float4* accumulator = nullptr;
    float4* colors = nullptr;
    LaunchShape shape{};
    tr_batch_info info{};

    Settings graphSettings{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    bool graphValid = false;
    cudaEvent_t evStart = nullptr, evStop = nullptr;
    bool timed = false;
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

void release(Batch* b)
{
    if (b->graphExec)
        cudaGraphExecDestroy(b->graphExec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    if (b->evStart)
        cudaEventDestroy(b->evStart);
    if (b->evStop)
        cudaEventDestroy(b->evStop);
    if (b->sceneArena)
        cudaFree(b->sceneArena);
    if (b->frameArena)
        cudaFree(b->frameArena);
    for (cudaEvent_t e : b->evFinal)
        if (e)
            cudaEventDestroy(e);
    if (b->evFork)
        cudaEventDestroy(b->evFork);
    for (cudaStream_t l : b->lanes)
        if (l)
            cudaStreamDestroy(l);
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

// Consecutive (item, sample) units into waves of at most `cap` paths.
void plan_waves(const std::vector<BatchItem>& items, uint64_t cap, std::vector<Wave>& waves,
                std::vector<BatchSegment>& segs)
{
    Wave w{};
    w.segmentOffset = 0;
    auto close = [&]() {
        if (w.segmentCount) {
            waves.push_back(w);
            w = Wave{};
            w.segmentOffset = uint32_t(segs.size());
        }
    };
    for (uint32_t i = 0; i < items.size(); ++i) {
        const uint64_t px = uint64_t(items[i].width) * items[i].height;
        uint32_t done = 0;
        while (done < items[i].spp) {
            uint64_t fit = (cap - w.paths) / px;
            if (fit == 0) {
                close();
                fit = cap / px;
            }
            const uint32_t k = uint32_t(std::min<uint64_t>(fit, items[i].spp - done));
            BatchSegment sg{};
            sg.pathBase = w.paths;
            sg.pixelBase = w.pixels;
            sg.item = i;
            sg.sampleBase = done;
            sg.pixels = uint32_t(px);
            sg.samples = k;
            segs.push_back(sg);
            w.segmentCount++;
            w.paths += uint32_t(k * px);
            w.pixels += uint32_t(px);
            done += k;
        }
    }
    close();
}

FrameView wave_view(const Batch* b, uint32_t w)
{
    FrameView f = b->frame[w % kWaveSets];
    const Wave& wv = b->waves[w];
    f.segments = b->segments + wv.segmentOffset;
    f.segmentCount = wv.segmentCount;
    f.pathCount = wv.paths;
    f.counters = b->counters + size_t(w) * kCounterWords;
    return f;
}

cudaError_t enqueue(Batch* b, const Settings& st, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(b->accumulator, 0, size_t(b->info.pixel_count) * sizeof(float4), s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(b->counters, 0, b->waves.size() * kCounterWords * sizeof(uint32_t), s);
    const Camera noCamera{};  // each path uses its item's camera
    if (e == cudaSuccess)
        e = cudaEventRecord(b->evFork, s);
    for (uint32_t k = 0; e == cudaSuccess && k < kWaveSets; ++k)
        e = cudaStreamWaitEvent(b->lanes[k], b->evFork, 0);
    for (uint32_t w = 0; e == cudaSuccess && w < b->waves.size(); ++w) {
        // a set's stream runs its waves in order, so a wave reuses the buffers of the
        // wave two before it only after that one finished
        cudaStream_t ls = b->lanes[w % kWaveSets];
        const FrameView f = wave_view(b, w);
        // the camera rays are made inside the first extend launch
        for (uint32_t bounce = 0; e == cudaSuccess && bounce < st.maxDepth; ++bounce) {
            e = launch_extend(b->scene, f, st, bounce, b->shape, ls, &noCamera);
            if (e == cudaSuccess)
                e = launch_shade(b->scene, f, st, bounce, b->shape, ls);
            if (e == cudaSuccess)
                e = launch_connect(b->scene, f, st, bounce, b->shape, ls);
        }
        // accumulator updates in wave order: an item split over two waves adds to the same pixels
        if (e == cudaSuccess && w > 0)
            e = cudaStreamWaitEvent(ls, b->evFinal[w - 1], 0);
        if (e == cudaSuccess)
            e = launch_batch_finalize(f, b->waves[w].pixels, ls);
        if (e == cudaSuccess)
            e = cudaEventRecord(b->evFinal[w], ls);
    }
    // the last wave's accumulator update follows every earlier one and its own wave
    if (e == cudaSuccess && !b->waves.empty())
        e = cudaStreamWaitEvent(s, b->evFinal[b->waves.size() - 1], 0);
    for (uint32_t k = 1; e == cudaSuccess && k < kWaveSets && k < b->waves.size(); ++k)
        e = cudaStreamWaitEvent(s, b->evFinal[b->waves.size() - 1 - k], 0);
    if (e == cudaSuccess)
        e = launch_batch_resolve(b->accumulator, b->colors, uint32_t(b->info.pixel_count), s);
    return e;
}

} // namespace

extern "C" {

tr_status tr_batch_create(const tr_config* config, const tr_batch_item* items, uint32_t count,
                          uint64_t wave_paths, void** out_batch)
{
    if (!config || !out_batch || !items || count == 0)
        return TR_ERR_INVALID_ARGUMENT;
    *out_batch = nullptr;
    if (config->abi_version != TR_ABI_VERSION)
        return TR_ERR_INVALID_ARGUMENT;
    const uint64_t cap = wave_paths ? wave_paths : kDefaultWavePaths;
    if (cap >= TR_MAX_PATHS)
        return TR_ERR_LIMIT;
    uint64_t pixels = 0, paths = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const tr_batch_item& it = items[i];
        if (!it.scene || it.width == 0 || it.height == 0 || it.spp == 0)
            return TR_ERR_INVALID_ARGUMENT;
        if (uint64_t(it.width) * it.height > cap)
            return TR_ERR_LIMIT;
        if (!validate_scene(*it.scene).empty() || it.scene->instance_count || it.scene->material_textures)
            return TR_ERR_INVALID_ARGUMENT;  // one-mesh untextured scenes only
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
    if (cudaStreamCreate(&b->stream) != cudaSuccess ||
        cudaEventCreate(&b->evStart) != cudaSuccess || cudaEventCreate(&b->evStop) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->evFork, cudaEventDisableTiming) != cudaSuccess)
        return bail(TR_ERR_CUDA);
    for (uint32_t k = 0; k < kWaveSets; ++k)
        if (cudaStreamCreateWithFlags(&b->lanes[k], cudaStreamNonBlocking) != cudaSuccess)
            return bail(TR_ERR_CUDA);

    const auto t0 = std::chrono::steady_clock::now();
    std::vector<ItemBuild> built = build_items(items, count, 3u);
    for (const ItemBuild& r : built)
        if (!r.error.empty())
            return bail(TR_ERR_INVALID_ARGUMENT);

    // concatenated host buffers with rebased indices
    std::vector<CwbvhNode> nodes;
    std::vector<float4> btris;
    std::vector<TriShade> tris;
    std::vector<uint32_t> matIdx;
    std::vector<Material> materials;
    std::vector<LightTri> lights;
    std::vector<AliasEntry> alias;
    b->items.resize(count);
    uint64_t pixelBase = 0, triTotal = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const ItemBuild& r = built[i];
        const uint32_t nodeBase = uint32_t(nodes.size());
        const uint32_t slotBase = uint32_t(btris.size() / 3);
        const uint32_t primBase = uint32_t(tris.size());
        const uint32_t matBase = uint32_t(materials.size());
        const uint32_t lightBase = uint32_t(lights.size());
        for (CwbvhNode n : r.bvh.nodes) {
            n.w[1].x += nodeBase;
            n.w[1].y += slotBase;
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
    std::vector<Wave> waves;
    std::vector<BatchSegment> segs;
    plan_waves(b->items, cap, waves, segs);
    const auto t1 = std::chrono::steady_clock::now();

    // scene arena
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + std::max<size_t>(bytes, 16));
        return o;
    };
    const size_t oNodes = take(nodes.size() * sizeof(CwbvhNode));
    const size_t oBTris = take(btris.size() * sizeof(float4));
    const size_t oTris = take(tris.size() * sizeof(TriShade));
    const size_t oMat = take(matIdx.size() * sizeof(uint32_t));
    const size_t oMats = take(materials.size() * sizeof(Material));
    const size_t oLights = take(lights.size() * sizeof(LightTri));
    const size_t oAlias = take(alias.size() * sizeof(AliasEntry));
    const size_t oXf = take(sizeof(identity));
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
        up(oNodes, nodes.data(), nodes.size() * sizeof(CwbvhNode)),
        up(oBTris, btris.data(), btris.size() * sizeof(float4)),
        up(oTris, tris.data(), tris.size() * sizeof(TriShade)),
        up(oMat, matIdx.data(), matIdx.size() * sizeof(uint32_t)),
        up(oMats, materials.data(), materials.size() * sizeof(Material)),
        up(oLights, lights.data(), lights.size() * sizeof(LightTri)),
        up(oAlias, alias.data(), alias.size() * sizeof(AliasEntry)),
        up(oXf, identity, sizeof(identity)),
    };
    for (cudaError_t x : es)
        if (x != cudaSuccess)
            return bail(TR_ERR_CUDA);
    SceneView& sv = b->scene;
    sv.nodes = reinterpret_cast<const CwbvhNode*>(sb + oNodes);
    sv.bvhTris = reinterpret_cast<const float4*>(sb + oBTris);
    sv.tris = reinterpret_cast<const TriShade*>(sb + oTris);
    sv.matIdx = reinterpret_cast<const uint32_t*>(sb + oMat);
    sv.materials = reinterpret_cast<const Material*>(sb + oMats);
    sv.lights = reinterpret_cast<const LightTri*>(sb + oLights);
    sv.alias = reinterpret_cast<const AliasEntry*>(sb + oAlias);
    sv.invTransforms = reinterpret_cast<const float4*>(sb + oXf);
    sv.nodeCount = uint32_t(nodes.size());
    sv.triCount = uint32_t(tris.size());

    // frame arena: wave buffers, batch accumulator and colors, tables
    uint32_t capPaths = 0;
    for (const Wave& w : waves)
        capPaths = std::max(capPaths, w.paths);
    const size_t capN = capPaths;
    off = 0;
    size_t oS0[kWaveSets], oS1[kWaveSets], oHits[kWaveSets], oShadow[kWaveSets], oRad[kWaveSets];
    const uint32_t sets = uint32_t(std::min<size_t>(kWaveSets, waves.size()));
    for (uint32_t k = 0; k < sets; ++k) {
        oS0[k] = take(3 * capN * sizeof(float4));
        oS1[k] = take(3 * capN * sizeof(float4));
        oHits[k] = take(capN * sizeof(uint4));
        oShadow[k] = take(3 * capN * sizeof(float4));
        oRad[k] = take(capN * sizeof(float4));
    }
    const size_t oAcc = take(pixels * sizeof(float4));
    const size_t oCol = take(pixels * sizeof(float4));
    const size_t oCnt = take(waves.size() * kCounterWords * sizeof(uint32_t));
    const size_t oSeg = take(segs.size() * sizeof(BatchSegment));
    const size_t oItems = take(b->items.size() * sizeof(BatchItem));
    const size_t oWords = take(2 * sizeof(uint32_t));
    const size_t oTrav = take(4 * sizeof(unsigned long long));
    e = cudaMalloc(&b->frameArena, off);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bail(e == cudaErrorMemoryAllocation ? TR_ERR_OUT_OF_MEMORY : TR_ERR_CUDA);
    }
    char* fb = static_cast<char*>(b->frameArena);
    if (cudaMemset(fb, 0, off) != cudaSuccess ||
        cudaMemcpy(fb + oSeg, segs.data(), segs.size() * sizeof(BatchSegment), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(fb + oItems, b->items.data(), b->items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice) !=
            cudaSuccess)
        return bail(TR_ERR_CUDA);
    FrameView f{};
    f.accumulator = reinterpret_cast<float4*>(fb + oAcc);
    f.colors = reinterpret_cast<float4*>(fb + oCol);
    f.albedo = nullptr;
    f.normals = nullptr;
    f.sampleCount = reinterpret_cast<uint32_t*>(fb + oWords);      // stays 0: samples are keyed per segment
    f.errorFlag = reinterpret_cast<uint32_t*>(fb + oWords) + 1;
    f.traversal = reinterpret_cast<unsigned long long*>(fb + oTrav);
    f.capacity = capPaths;
    f.resX = 1;
    f.resY = 1;
    f.items = reinterpret_cast<const BatchItem*>(fb + oItems);
    for (uint32_t k = 0; k < kWaveSets; ++k) {
        const uint32_t j = k < sets ? k : 0u;
        b->frame[k] = f;
        b->frame[k].state[0] = reinterpret_cast<float4*>(fb + oS0[j]);
        b->frame[k].state[1] = reinterpret_cast<float4*>(fb + oS1[j]);
        b->frame[k].hits = reinterpret_cast<uint4*>(fb + oHits[j]);
        b->frame[k].shadow = reinterpret_cast<float4*>(fb + oShadow[j]);
        b->frame[k].radiance = reinterpret_cast<float4*>(fb + oRad[j]);
    }
    b->evFinal.assign(waves.size(), nullptr);
    for (cudaEvent_t& ev : b->evFinal)
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
            return bail(TR_ERR_CUDA);
    b->segments = reinterpret_cast<BatchSegment*>(fb + oSeg);
    b->counters = reinterpret_cast<uint32_t*>(fb + oCnt);
    b->accumulator = f.accumulator;
    b->colors = f.colors;
    b->waves = waves;
    b->shape = default_launch_shape(b->device, capPaths);
    const auto t2 = std::chrono::steady_clock::now();

    tr_batch_info& in = b->info;
    in.item_count = count;
    in.wave_count = uint32_t(waves.size());
    in.path_count = paths;
    in.pixel_count = pixels;
    in.triangle_count = triTotal;
    in.device_bytes = sceneBytes + off;
    in.wave_paths = capPaths;
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
    Batch* b = static_cast<Batch*>(batch);
    *out = b->info;
    out->launches = uint32_t(b->waves.size()) * (1u + 3u * b->lastSettings.maxDepth) + 1u;
    return TR_OK;
}

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
    TR_BCUDA(b, cudaEventRecord(b->evStart, s));
    if (use_graph && !(st.flags & TR_FLAG_COUNT_TRAVERSAL)) {
        if (!b->graphValid || std::memcmp(&st, &b->graphSettings, sizeof(Settings)) != 0) {
            if (b->graphExec)
                cudaGraphExecDestroy(b->graphExec);
            if (b->graph)
                cudaGraphDestroy(b->graph);
            b->graphExec = nullptr;
            b->graph = nullptr;
            b->graphValid = false;
            TR_BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            const cudaError_t ec = enqueue(b, st, b->stream);
            cudaGraph_t g = nullptr;
            const cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
            if (ec != cudaSuccess || ee != cudaSuccess) {
                if (g)
                    cudaGraphDestroy(g);
                return cuda_fail(b, ec != cudaSuccess ? ec : ee, "batch graph capture");
            }
            b->graph = g;
            TR_BCUDA(b, cudaGraphInstantiate(&b->graphExec, g, 0));
            b->graphSettings = st;
            b->graphValid = true;
        }
        TR_BCUDA(b, cudaGraphLaunch(b->graphExec, s));
    } else {
        if (st.flags & TR_FLAG_COUNT_TRAVERSAL)
            TR_BCUDA(b, cudaMemsetAsync(b->frame[0].traversal, 0, 4 * sizeof(unsigned long long), s));
        TR_BCUDA(b, enqueue(b, st, s));
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
    std::vector<uint32_t> cnt(b->waves.size() * kCounterWords);
    TR_BCUDA(b, cudaMemcpy(cnt.data(), b->counters, cnt.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    uint32_t err = 0;
    unsigned long long trav[4] = {0, 0, 0, 0};
    TR_BCUDA(b, cudaMemcpy(&err, b->frame[0].errorFlag, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    TR_BCUDA(b, cudaMemcpy(trav, b->frame[0].traversal, sizeof(trav), cudaMemcpyDeviceToHost));
    tr_batch_statistics s{};
    for (size_t w = 0; w < b->waves.size(); ++w) {
        const uint32_t* c = cnt.data() + w * kCounterWords;
        for (uint32_t bounce = 0; bounce < b->lastSettings.maxDepth; ++bounce) {
            s.extend_rays += bounce == 0 ? b->waves[w].paths : c[bounce];
            s.shadow_rays += c[kShadowCounterBase + bounce];
            s.hit_rays += c[kHitCounterBase + bounce];
        }
    }
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
