// C ABI of the wavefront path tracer: context, scene upload, wavefront
// buffers, per-stage launches, CUDA-graph frame loop, statistics.
//
// Mirrors the reference's DeviceRenderer (Tracer/Renderer/DeviceRenderer.cpp)
// and Renderer upload path (Tracer/Renderer/Renderer.cpp:442-527), with
// status codes instead of CUDA_CHECK -> FatalError -> exit
// (Tracer/CUDA/CudaError.cpp:13-25), scene pointers passed as kernel
// parameters instead of __constant__ symbols (Tracer/CUDA/GPU/CudaGlobals.h),
// and no host round trip per bounce (the reference downloads the ray counters
// after every shade, DeviceRenderer.cpp:255-257).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/trayracer.h"
#include "tr_api_internal.h"
#include "tr_accel.h"
#include "tr_bvh.h"
#include "tr_continuous.h"
#include "tr_kernels.h"
#include "tr_sky.h"
#include "tr_scene.h"

namespace {

using namespace tr;

struct DeviceArena {
    void* base = nullptr;
    size_t bytes = 0;
    void release()
    {
        if (base)
            cudaFree(base);
        base = nullptr;
        bytes = 0;
    }
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// A copy of a scene's meshes and instances that outlives tr_scene_upload's
// arguments (the BVH is rebuilt from it when the leaf size is tuned).
struct OwnedGeometry {
    std::vector<std::vector<float>> positions;
    std::vector<std::vector<uint32_t>> indices;
    std::vector<tr_mesh_desc> meshes;
    std::vector<tr_instance_desc> instances;
    tr_scene_desc desc{};

    void assign(const tr_scene_desc& d)
    {
        const uint32_t n = scene_mesh_count(d);
        positions.assign(n, {});
        indices.assign(n, {});
        meshes.assign(n, tr_mesh_desc{});
        for (uint32_t i = 0; i < n; ++i) {
            const tr_mesh_desc& m = scene_mesh(d, i);
            positions[i].assign(m.positions, m.positions + size_t(m.vertex_count) * 3);
            indices[i].assign(m.indices, m.indices + size_t(m.triangle_count) * 3);
            meshes[i] = tr_mesh_desc{positions[i].data(), nullptr, nullptr, m.vertex_count, m.triangle_count,
                                     indices[i].data(), nullptr};
        }
        instances.assign(d.instances, d.instances + d.instance_count);
        desc = tr_scene_desc{};
        desc.instance_count = d.instance_count;
        if (d.instance_count) {
            desc.meshes = meshes.data();
            desc.mesh_count = n;
            desc.instances = instances.data();
        } else {
            desc.mesh = meshes.data();
        }
    }
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string lastError;

    // scene
    bool hasScene = false;
    DeviceArena sceneArena;
    DeviceArena bvhArena;          // nodes + traversal triangles (rebuilt when the leaf size is tuned)
    OwnedGeometry geom;            // host copy of the meshes and instances, for BVH rebuilds
    std::vector<uint32_t> meshTriBase;
    uint32_t leafSize = 3;
    uint32_t nodeMode = 0;         // tr_tuning.bvh_nodes: 0 auto, 1 fp32, 2 quantized
    tr_tuning tuning{};
    SceneView scene{};
    tr_scene_info info{};
    // host copies kept for material updates without a BVH rebuild
    std::vector<LightTri> hostLights;
    std::vector<uint32_t> hostMatIdx;
    uint32_t materialCount = 0;

    // settings / camera
    Settings settings{};
    Camera camera{};
    bool hasCamera = false;

    // frame
    uint32_t width = 0, height = 0;
    DeviceArena frameArena;
    FrameView frame{};
    SortView sort{};               // material sort of the hit queue (keys/order in the frame arena, bins in the scene arena)
    DeviceArena adjointArena;      // path-replay scratch, allocated by the first tr_adjoint_frame of a frame size
    AdjointView adjoint{};
    uint32_t* adjointCounters = nullptr;
    size_t frameCapacity = 0;
    uint32_t frameW = 0, frameH = 0, frameMs = 0;
    LaunchShape shape{};
    uint32_t sampleCount = 0;
    float* pickResult = nullptr;       // 9 words of the frame arena (tr_pick_ray)

    // textures of the scene: one CUDA array and texture object each, and the
    // per-material slots as uploaded (kept to rewrite their emissive colour)
    std::vector<cudaArray_t> texArrays;
    std::vector<cudaTextureObject_t> texObjects;
    std::vector<TexSlots> texSlotsHost;

    // timing
    cudaEvent_t evStart = nullptr, evGenerate = nullptr, evFinal = nullptr;
    // captured frames trace bounce b's shadow rays on this stream while bounce
    // b + 1's extend rays run on the frame's stream (fork / join)
    cudaStream_t side = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    cudaEvent_t evExtend[TR_MAX_DEPTH] = {}, evShade[TR_MAX_DEPTH] = {}, evConnect[TR_MAX_DEPTH] = {};
    bool timedFrame = false;
    uint32_t timedDepth = 0;
    cudaStream_t lastStream = nullptr;

    // graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    bool graphValid = false;

    // tr_render_samples: per-sample radiance, the one item and the iteration
    // state of the continuous wavefront, and its graph (per sample count)
    DeviceArena samplesArena;
    uint64_t samplesCapacity = 0;      // per-sample radiance entries the arena holds
    float4* sampleRadiance = nullptr;
    BatchItem* samplesItem = nullptr;
    BatchState* samplesState = nullptr;
    BatchItem samplesItemHost{};       // what samplesItem holds
    bool samplesItemValid = false;
    cudaGraph_t samplesGraph = nullptr;
    cudaGraphExec_t samplesExec = nullptr;
    uint32_t samplesGraphSpp = 0;
    bool lastSamples = false;          // the last render was tr_render_samples' continuous wavefront
    uint32_t lastSamplesPaths = 0;
    bool samplesTimed = false;         // ... rendered eagerly, with its stage times
    StageTimes samplesTimes{};

    // frames rendered by tr_render_frame_noalloc: the launch shape for their
    // capacity and tuning, and whether the last frame was one of them
    LaunchShape noallocShape{};
    uint32_t noallocShapeCap = 0;
    tr_tuning noallocShapeTuning{};
    bool lastFrameNoalloc = false;
    uint32_t noallocPaths = 0;

    // render mode (RenderModes; debug modes run the reference's other shade kernels)
    uint32_t renderMode = kModePathTracing;
    uint32_t renderFlags = 0;
    float aoDist = 1.f;
    float zDepthMax = 1.f;
};

tr_status fail(Context* c, tr_status st, const std::string& msg)
{
    if (c)
        c->lastError = msg;
    return st;
}

tr_status cuda_fail(Context* c, cudaError_t e, const char* what)
{
    const bool sticky = e == cudaErrorIllegalAddress || e == cudaErrorLaunchFailure ||
                        e == cudaErrorIllegalInstruction || e == cudaErrorMisalignedAddress ||
                        e == cudaErrorHardwareStackError || e == cudaErrorAssert;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(c, TR_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
    }
    return fail(c, sticky ? TR_ERR_DEVICE_FAULT : TR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define TR_CUDA(ctx, call)                                  \
    do {                                                    \
        const cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess)                              \
            return cuda_fail((ctx), e_, #call);             \
    } while (0)

cudaStream_t pick_stream(Context* c, void* s) { return s ? static_cast<cudaStream_t>(s) : c->stream; }

void invalidate_graph(Context* c)
{
    if (c->graphExec)
        cudaGraphExecDestroy(c->graphExec);
    if (c->graph)
        cudaGraphDestroy(c->graph);
    c->graphExec = nullptr;
    c->graph = nullptr;
    c->graphValid = false;
    if (c->samplesExec)
        cudaGraphExecDestroy(c->samplesExec);
    if (c->samplesGraph)
        cudaGraphDestroy(c->samplesGraph);
    c->samplesExec = nullptr;
    c->samplesGraph = nullptr;
    c->samplesGraphSpp = 0;
    c->samplesItemValid = false;
}

void release_textures(Context* c)
{
    for (cudaTextureObject_t t : c->texObjects)
        cudaDestroyTextureObject(t);
    for (cudaArray_t a : c->texArrays)
        cudaFreeArray(a);
    c->texObjects.clear();
    c->texArrays.clear();
    c->texSlotsHost.clear();
}

// A context's texture: owned by the context from here on.
tr_status upload_texture(Context* c, const tr_texture_desc& t)
{
    cudaArray_t arr = nullptr;
    cudaTextureObject_t obj = 0;
    const cudaError_t e = create_texture(t, &arr, &obj);
    if (arr)
        c->texArrays.push_back(arr);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "create_texture");
    c->texObjects.push_back(obj);
    return TR_OK;
}

// Uploads the acceleration structures into their own arena and points the
// scene view at them.
tr_status upload_bvh(Context* c, const SceneAccel& acc)
{
    const bool quant = quantized_nodes(acc.nodes.size() + acc.tlasNodes.size(), c->nodeMode, !acc.tlasNodes.empty());
    const std::vector<QuantNode> qnodes = quant ? quantize_nodes(acc.nodes) : std::vector<QuantNode>{};
    const std::vector<QuantNode> qtlas = quant ? quantize_nodes(acc.tlasNodes) : std::vector<QuantNode>{};
    const void* nodeSrc = quant ? static_cast<const void*>(qnodes.data()) : static_cast<const void*>(acc.nodes.data());
    const void* tlasSrc = quant ? static_cast<const void*>(qtlas.data()) : static_cast<const void*>(acc.tlasNodes.data());
    const size_t nodeSize = quant ? sizeof(QuantNode) : sizeof(WideNode);
    const size_t nodeBytes = acc.nodes.size() * nodeSize;
    const size_t tlasBytes = acc.tlasNodes.size() * nodeSize;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + std::max<size_t>(bytes, 16));
        return o;
    };
    const size_t oN = take(nodeBytes);
    const size_t oT = take(acc.tris.size() * sizeof(float4));
    const size_t oTl = take(tlasBytes);
    const size_t oTi = take(acc.tlasInst.size() * sizeof(uint32_t));
    const size_t oIi = take(acc.instInfo.size() * sizeof(uint2));
    void* base = nullptr;
    cudaError_t e = cudaMalloc(&base, off);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "cudaMalloc(bvh)");
    char* b = static_cast<char*>(base);
    auto up = [&](size_t o, const void* src, size_t bytes) {
        return bytes ? cudaMemcpy(b + o, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
    };
    const cudaError_t es[] = {
        up(oN, nodeSrc, nodeBytes),
        up(oT, acc.tris.data(), acc.tris.size() * sizeof(float4)),
        up(oTl, tlasSrc, tlasBytes),
        up(oTi, acc.tlasInst.data(), acc.tlasInst.size() * sizeof(uint32_t)),
        up(oIi, acc.instInfo.data(), acc.instInfo.size() * sizeof(uint2)),
    };
    for (cudaError_t x : es)
        if (x != cudaSuccess) {
            cudaFree(base);
            return cuda_fail(c, x, "cudaMemcpy(bvh)");
        }
    c->bvhArena.release();
    c->bvhArena.base = base;
    c->bvhArena.bytes = off;
    c->scene.nodes = b + oN;
    c->scene.quantNodes = quant ? 1u : 0u;
    c->scene.bvhTris = reinterpret_cast<const float4*>(b + oT);
    c->scene.nodeCount = uint32_t(acc.nodes.size());
    const bool twoLevel = !acc.tlasNodes.empty();
    c->scene.tlasNodes = twoLevel ? static_cast<const void*>(b + oTl) : nullptr;
    c->scene.tlasInst = twoLevel ? reinterpret_cast<const uint32_t*>(b + oTi) : nullptr;
    c->scene.instInfo = twoLevel ? reinterpret_cast<const uint2*>(b + oIi) : nullptr;
    c->info.bvh_node_count = uint32_t(acc.nodes.size() + acc.tlasNodes.size());
    return TR_OK;
}

// Rebuilds the BVH from the host copy of the geometry with another leaf size
// or node layout.
tr_status rebuild_bvh(Context* c, uint32_t leafSize, uint32_t nodeMode)
{
    if (leafSize == c->leafSize && nodeMode == c->nodeMode)
        return TR_OK;
    const uint32_t oldMode = c->nodeMode;
    c->nodeMode = nodeMode;
    BvhBuildOptions opt;
    opt.maxLeafSize = leafSize;
    const SceneAccel wide = build_accel(c->geom.desc, c->meshTriBase, opt);
    if (c->stream)
        cudaStreamSynchronize(c->stream);
    cudaDeviceSynchronize();
    invalidate_graph(c);
    const tr_status st = upload_bvh(c, wide);
    if (st == TR_OK)
        c->leafSize = leafSize;
    else
        c->nodeMode = oldMode;
    return st;
}

tr_status ensure_frame(Context* c)
{
    if (c->width == 0 || c->height == 0)
        return fail(c, TR_ERR_NOT_READY, "resolution not set (tr_resize)");
    const uint64_t wh = uint64_t(c->width) * c->height;
    const uint64_t paths = wh * c->settings.multiSample;
    if (paths == 0 || paths >= TR_MAX_PATHS)
        return fail(c, TR_ERR_LIMIT, "paths in flight (width*height*multi_sample) must be in [1, 2^28)");
    if (c->frameArena.base && c->frameW == c->width && c->frameH == c->height && c->frameMs == c->settings.multiSample)
        return TR_OK;

    invalidate_graph(c);
    c->frameArena.release();
    c->adjointArena.release();
    c->samplesArena.release();
    c->samplesCapacity = 0;
    const size_t cap = size_t(paths);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    const size_t oState0 = take(3 * cap * sizeof(float4));
    const size_t oState1 = take(3 * cap * sizeof(float4));
    const size_t oHits = take(cap * sizeof(uint4));
    const size_t oShadow = take(3 * cap * sizeof(float4));
    const size_t oRad = take(cap * sizeof(float4));
    const size_t oAcc = take(wh * sizeof(float4));
    const size_t oAlb = take(wh * sizeof(float4));
    const size_t oNrm = take(wh * sizeof(float4));
    const size_t oCol = take(wh * sizeof(float4));
    const size_t oCnt = take(kCounterWords * sizeof(uint32_t));
    const size_t oSc = take(sizeof(uint32_t));
    const size_t oErr = take(sizeof(uint32_t));
    const size_t oTrav = take(kTraversalCounters * sizeof(unsigned long long));
    const size_t oKeys = take(cap * sizeof(uint32_t));
    const size_t oOrder = take(cap * sizeof(uint32_t));
    const size_t oPick = take(16 * sizeof(float));
    void* base = nullptr;
    const cudaError_t e = cudaMalloc(&base, off);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "cudaMalloc(frame buffers)");
    c->frameArena.base = base;
    c->frameArena.bytes = off;
    char* b = static_cast<char*>(base);
    FrameView& f = c->frame;
    f.state[0] = reinterpret_cast<float4*>(b + oState0);
    f.state[1] = reinterpret_cast<float4*>(b + oState1);
    f.hits = reinterpret_cast<uint4*>(b + oHits);
    f.shadow = reinterpret_cast<float4*>(b + oShadow);
    f.radiance = reinterpret_cast<float4*>(b + oRad);
    f.accumulator = reinterpret_cast<float4*>(b + oAcc);
    f.albedo = reinterpret_cast<float4*>(b + oAlb);
    f.normals = reinterpret_cast<float4*>(b + oNrm);
    f.colors = reinterpret_cast<float4*>(b + oCol);
    f.counters = reinterpret_cast<uint32_t*>(b + oCnt);
    f.sampleCount = reinterpret_cast<uint32_t*>(b + oSc);
    f.errorFlag = reinterpret_cast<uint32_t*>(b + oErr);
    f.traversal = reinterpret_cast<unsigned long long*>(b + oTrav);
    c->sort.keys = reinterpret_cast<uint32_t*>(b + oKeys);
    c->sort.order = reinterpret_cast<uint32_t*>(b + oOrder);
    c->pickResult = reinterpret_cast<float*>(b + oPick);
    f.capacity = uint32_t(cap);
    f.resX = c->width;
    f.resY = c->height;
    f.pathCount = uint32_t(paths);
    TR_CUDA(c, cudaMemset(base, 0, off));
    c->frameCapacity = cap;
    c->frameW = c->width;
    c->frameH = c->height;
    c->frameMs = c->settings.multiSample;
    c->sampleCount = 0;
    c->shape = tuned_launch_shape(c->device, uint32_t(cap), c->tuning);
    f.hitOrder = c->shape.sortHits ? c->sort.order : nullptr;
    return TR_OK;
}

tr_status check_ready(Context* c)
{
    if (!c->hasScene)
        return fail(c, TR_ERR_NO_SCENE, "no scene uploaded");
    if (!c->hasCamera)
        return fail(c, TR_ERR_NOT_READY, "camera not set");
    return ensure_frame(c);
}

tr_status enqueue_begin(Context* c, cudaStream_t s)
{
    TR_CUDA(c, cudaMemsetAsync(c->frame.counters, 0, kCounterWords * sizeof(uint32_t), s));
    return TR_OK;
}

tr_status enqueue_frame(Context* c, cudaStream_t s, bool timed)
{
    tr_status st = enqueue_begin(c, s);
    if (st != TR_OK)
        return st;
    if (timed)
        TR_CUDA(c, cudaEventRecord(c->evStart, s));
    if (c->renderMode != kModePathTracing) {
        Settings st = c->settings;
        st.renderMode = c->renderMode;
        st.renderFlags = c->renderFlags;
        st.aoDist = c->aoDist;
        st.zDepthMax = c->zDepthMax;
        TR_CUDA(c, launch_generate(c->frame, c->camera, st, s));
        if (timed)
            TR_CUDA(c, cudaEventRecord(c->evGenerate, s));
        for (uint32_t b = 0; b < st.maxDepth; ++b) {
            TR_CUDA(c, launch_debug_bounce(c->scene, c->frame, c->camera, st, b, c->shape, s));
            if (timed) {
                TR_CUDA(c, cudaEventRecord(c->evExtend[b], s));
                TR_CUDA(c, cudaEventRecord(c->evShade[b], s));
                TR_CUDA(c, cudaEventRecord(c->evConnect[b], s));
            }
        }
        TR_CUDA(c, launch_finalize(c->frame, c->settings, s));
        if (timed)
            TR_CUDA(c, cudaEventRecord(c->evFinal, s));
        return TR_OK;
    }
    // default sampling mode: the camera rays are made inside the first extend launch
    const bool fused = (c->settings.flags & TR_FLAG_REFERENCE_SAMPLING) == 0;
    if (!fused)
        TR_CUDA(c, launch_generate(c->frame, c->camera, c->settings, s));
    if (timed)
        TR_CUDA(c, cudaEventRecord(c->evGenerate, s));
    // Untimed (captured) frames overlap bounce b's connect with bounce b + 1's
    // extend: connect reads the shadow queue and adds to the radiance of paths
    // in flight, extend reads the extend queue and writes the hit queue, so they
    // share nothing; shade b + 1 (which rewrites the shadow queue and adds
    // emission to the same radiance) waits for both. Not with a sky: extend
    // adds the sky to the radiance of missed paths. Timed frames keep the
    // stages in sequence for their per-stage events.
    const bool overlap = !timed && !c->scene.sky.enabled;
    for (uint32_t b = 0; b < c->settings.maxDepth; ++b) {
        TR_CUDA(c, launch_extend(c->scene, c->frame, c->settings, b, c->shape, s, fused ? &c->camera : nullptr));
        if (c->shape.sortHits)
            TR_CUDA(c, launch_sort_hits(c->scene, c->frame, c->sort, b, c->shape, s));
        if (timed)
            TR_CUDA(c, cudaEventRecord(c->evExtend[b], s));
        if (overlap && b > 0)
            TR_CUDA(c, cudaStreamWaitEvent(s, c->evJoin, 0));
        TR_CUDA(c, launch_shade(c->scene, c->frame, c->settings, b, c->shape, s));
        if (timed)
            TR_CUDA(c, cudaEventRecord(c->evShade[b], s));
        if (overlap) {
            TR_CUDA(c, cudaEventRecord(c->evFork, s));
            TR_CUDA(c, cudaStreamWaitEvent(c->side, c->evFork, 0));
            TR_CUDA(c, launch_connect(c->scene, c->frame, c->settings, b, c->shape, c->side));
            TR_CUDA(c, cudaEventRecord(c->evJoin, c->side));
        } else {
            TR_CUDA(c, launch_connect(c->scene, c->frame, c->settings, b, c->shape, s));
        }
        if (timed)
            TR_CUDA(c, cudaEventRecord(c->evConnect[b], s));
    }
    if (overlap)
        TR_CUDA(c, cudaStreamWaitEvent(s, c->evJoin, 0));
    TR_CUDA(c, launch_finalize(c->frame, c->settings, s));
    if (timed)
        TR_CUDA(c, cudaEventRecord(c->evFinal, s));
    return TR_OK;
}

} // namespace

namespace tr {

tr_status context_views(void* ctx, ContextViews* out)
{
    if (!ctx || !out)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (!c->hasScene)
        return fail(c, TR_ERR_NO_SCENE, "no scene uploaded");
    if (!c->hasCamera)
        return fail(c, TR_ERR_NOT_READY, "camera not set");
    if (c->width == 0 || c->height == 0)
        return fail(c, TR_ERR_NOT_READY, "resolution not set (tr_resize)");
    out->device = c->device;
    out->stream = c->stream;
    out->scene = c->scene;
    out->camera = c->camera;
    out->settings = c->settings;
    out->width = c->width;
    out->height = c->height;
    out->renderMode = c->renderMode;
    return TR_OK;
}

tr_status context_launch_shape(void* ctx, uint32_t capacity, LaunchShape* out)
{
    if (!ctx || !out)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (c->noallocShapeCap != capacity || std::memcmp(&c->noallocShapeTuning, &c->tuning, sizeof(tr_tuning)) != 0) {
        c->noallocShape = tuned_launch_shape(c->device, capacity, c->tuning);
        c->noallocShape.sortHits = 0;
        c->noallocShapeCap = capacity;
        c->noallocShapeTuning = c->tuning;
    }
    *out = c->noallocShape;
    return TR_OK;
}

void context_note_noalloc_frame(void* ctx, uint32_t paths)
{
    Context* c = static_cast<Context*>(ctx);
    c->lastFrameNoalloc = true;
    c->lastSamples = false;
    c->noallocPaths = paths;
    c->timedFrame = false;
}

tr_status context_fail(void* ctx, tr_status st, const std::string& msg)
{
    return fail(static_cast<Context*>(ctx), st, msg);
}

bool convert_camera(const tr_camera& cam, Camera* out, std::string* err)
{
    Camera k{};
    k.pos = make_float3(cam.position[0], cam.position[1], cam.position[2]);
    k.side = make_float3(cam.side[0], cam.side[1], cam.side[2]);
    k.up = make_float3(cam.up[0], cam.up[1], cam.up[2]);
    k.forward = make_float3(cam.forward[0], cam.forward[1], cam.forward[2]);
    k.aperture = cam.aperture;
    k.distortion = cam.distortion;
    k.focalDist = cam.focal_dist;
    k.fov = cam.fov;
    k.bokehSideCount = cam.bokeh_side_count;
    k.bokehRotation = cam.bokeh_rotation;
    k.tanFov2 = tanf(cam.fov / 2.0f);
    if (!(cam.fov > 0.f && cam.fov < 3.14159f) || !(cam.focal_dist > 0.f)) {
        *err = "camera fov must be in (0, pi) and focal_dist > 0";
        return false;
    }
    *out = k;
    return true;
}

bool convert_settings(const tr_kernel_settings& s, Settings* out, std::string* err)
{
    if (s.max_depth == 0 || s.max_depth > TR_MAX_DEPTH) {
        *err = "multi_sample must be >= 1 and max_depth in [1, 16]";
        return false;
    }
    if (!(s.ray_epsilon >= 0.f)) {
        *err = "ray_epsilon must be >= 0";
        return false;
    }
    Settings k{};
    k.multiSample = s.multi_sample;
    k.maxDepth = s.max_depth;
    k.seed = s.seed;
    k.rayEpsilon = s.ray_epsilon;
    k.rrStart = s.rr_start;
    k.flags = s.flags;
    k.maxColor = s.max_color > 0.f ? s.max_color : 10.f;
    k.renderMode = kModePathTracing;
    k.aoDist = 1.f;
    k.zDepthMax = 1.f;
    k.stepLimit = s.traversal_step_limit ? s.traversal_step_limit : kMaxTraversalSteps;
    *out = k;
    return true;
}

} // namespace tr

namespace tr {
// Texture::Upload (Texture.cpp:83-139): RGBA binary16 texels in a CUDA array,
// sampled with bilinear filtering, wrap addressing and normalised coordinates
// (the same texture description as the reference's, so a texel fetch filters
// the same way).
cudaError_t create_texture(const tr_texture_desc& t, cudaArray_t* arrOut, cudaTextureObject_t* objOut)
{
    *arrOut = nullptr;
    *objOut = 0;
    const cudaChannelFormatDesc cd = cudaCreateChannelDescHalf4();
    cudaArray_t arr = nullptr;
    cudaError_t e = cudaMallocArray(&arr, &cd, t.width, t.height);
    if (e != cudaSuccess)
        return e;
    *arrOut = arr;
    const size_t pitch = size_t(t.width) * 4 * sizeof(uint16_t);
    e = cudaMemcpy2DToArray(arr, 0, 0, t.texels, pitch, pitch, t.height, cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
        return e;
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td{};
    td.addressMode[0] = cudaAddressModeWrap;
    td.addressMode[1] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    return cudaCreateTextureObject(objOut, &rd, &td, nullptr);
}
} // namespace tr

extern "C" {

const char* tr_status_string(tr_status status)
{
    switch (status) {
    case TR_OK: return "ok";
    case TR_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TR_ERR_OUT_OF_MEMORY: return "out of memory";
    case TR_ERR_CUDA: return "CUDA error";
    case TR_ERR_NO_SCENE: return "no scene";
    case TR_ERR_NOT_READY: return "not ready";
    case TR_ERR_LIMIT: return "limit exceeded";
    case TR_ERR_DEVICE_FAULT: return "device fault";
    }
    return "unknown status";
}

const char* tr_last_error(void* ctx)
{
    return ctx ? static_cast<Context*>(ctx)->lastError.c_str() : "null context";
}

tr_status tr_create(const tr_config* config, void** out_ctx)
{
    if (!out_ctx)
        return TR_ERR_INVALID_ARGUMENT;
    *out_ctx = nullptr;
    const int device = config ? config->device : 0;
    if (config && config->abi_version != TR_ABI_VERSION)
        return TR_ERR_INVALID_ARGUMENT;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return TR_ERR_CUDA;
    }
    if (device < 0 || device >= count)
        return TR_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess)
        return TR_ERR_CUDA;
    Context* c = new (std::nothrow) Context();
    if (!c)
        return TR_ERR_OUT_OF_MEMORY;
    c->device = device;
    c->settings.multiSample = 1;
    c->settings.maxDepth = TR_MAX_DEPTH;
    c->settings.seed = 0;
    c->settings.rayEpsilon = kEpsilon;
    c->settings.rrStart = 1;
    c->settings.flags = 0;
    c->settings.maxColor = 10.f;
    bool ok = cudaStreamCreate(&c->stream) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&c->evFork, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&c->evJoin, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreate(&c->evStart) == cudaSuccess && cudaEventCreate(&c->evGenerate) == cudaSuccess &&
         cudaEventCreate(&c->evFinal) == cudaSuccess;
    for (uint32_t i = 0; ok && i < TR_MAX_DEPTH; ++i)
        ok = cudaEventCreate(&c->evExtend[i]) == cudaSuccess && cudaEventCreate(&c->evShade[i]) == cudaSuccess &&
             cudaEventCreate(&c->evConnect[i]) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        tr_destroy(c);
        return TR_ERR_CUDA;
    }
    *out_ctx = c;
    return TR_OK;
}

tr_status tr_destroy(void* ctx)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    cudaSetDevice(c->device);
    if (c->stream)
        cudaStreamSynchronize(c->stream);
    invalidate_graph(c);
    c->sceneArena.release();
    c->bvhArena.release();
    c->frameArena.release();
    c->adjointArena.release();
    c->samplesArena.release();
    release_textures(c);
    cudaEvent_t* evs[] = {&c->evStart, &c->evGenerate, &c->evFinal, &c->evFork, &c->evJoin};
    for (cudaEvent_t* e : evs)
        if (*e)
            cudaEventDestroy(*e);
    for (uint32_t i = 0; i < TR_MAX_DEPTH; ++i) {
        if (c->evExtend[i]) cudaEventDestroy(c->evExtend[i]);
        if (c->evShade[i]) cudaEventDestroy(c->evShade[i]);
        if (c->evConnect[i]) cudaEventDestroy(c->evConnect[i]);
    }
    if (c->side)
        cudaStreamDestroy(c->side);
    if (c->stream)
        cudaStreamDestroy(c->stream);
    delete c;
    return TR_OK;
}

tr_status tr_scene_upload(void* ctx, const tr_scene_desc* desc)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (!desc)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "null scene description");
    const std::string err = validate_scene(*desc);
    if (!err.empty())
        return fail(c, TR_ERR_INVALID_ARGUMENT, err);
    cudaSetDevice(c->device);

    const auto t0 = std::chrono::steady_clock::now();
    FlatScene fs = flatten_scene(*desc);
    BvhBuildOptions opt;
    opt.maxLeafSize = desc->bvh_leaf_size ? desc->bvh_leaf_size : 3u;
    opt.threads = desc->build_threads;
    const SceneAccel wide = build_accel(*desc, fs.meshTriBase, opt);
    const uint32_t triCount = uint32_t(fs.tris.size());
    const auto t1 = std::chrono::steady_clock::now();

    // one arena for the shading buffers, one for the BVH
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + std::max<size_t>(bytes, 16));
        return o;
    };
    const size_t oTris = take(fs.tris.size() * sizeof(TriShade));
    const size_t oMat = take(fs.matIdx.size() * sizeof(uint32_t));
    const size_t oMats = take(fs.materials.size() * sizeof(Material));
    const size_t oLights = take(fs.lights.size() * sizeof(LightTri));
    const size_t oAlias = take(fs.alias.size() * sizeof(AliasEntry));
    const size_t oXf = take(fs.invTransforms.size() * sizeof(float4));
    const size_t oBins = take(2 * size_t(desc->material_count) * sizeof(uint32_t));  // sort counts + cursors
    const size_t oTex = take(fs.texSlots.size() * sizeof(TexSlots));

    if (c->stream)
        cudaStreamSynchronize(c->stream);
    invalidate_graph(c);
    c->sceneArena.release();
    c->bvhArena.release();
    release_textures(c);
    c->hasScene = false;
    if (!fs.texSlots.empty()) {
        for (uint32_t i = 0; i < desc->texture_count; ++i) {
            const tr_status ts = upload_texture(c, desc->textures[i]);
            if (ts != TR_OK) {
                release_textures(c);
                return ts;
            }
        }
        for (TexSlots& slot : fs.texSlots)
            for (uint32_t p = 0; p < TR_PROP_COUNT; ++p)
                if (slot.tex[p])
                    slot.tex[p] = c->texObjects[size_t(slot.tex[p] - 1u)];
    }
    void* base = nullptr;
    cudaError_t e = cudaMalloc(&base, off);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "cudaMalloc(scene)");
    c->sceneArena.base = base;
    c->sceneArena.bytes = off;
    char* b = static_cast<char*>(base);
    auto up = [&](size_t o, const void* src, size_t bytes) -> cudaError_t {
        if (bytes == 0)
            return cudaSuccess;
        return cudaMemcpy(b + o, src, bytes, cudaMemcpyHostToDevice);
    };
    const cudaError_t es[] = {
        up(oTris, fs.tris.data(), fs.tris.size() * sizeof(TriShade)),
        up(oMat, fs.matIdx.data(), fs.matIdx.size() * sizeof(uint32_t)),
        up(oMats, fs.materials.data(), fs.materials.size() * sizeof(Material)),
        up(oLights, fs.lights.data(), fs.lights.size() * sizeof(LightTri)),
        up(oAlias, fs.alias.data(), fs.alias.size() * sizeof(AliasEntry)),
        up(oXf, fs.invTransforms.data(), fs.invTransforms.size() * sizeof(float4)),
        up(oTex, fs.texSlots.data(), fs.texSlots.size() * sizeof(TexSlots)),
    };
    for (cudaError_t x : es)
        if (x != cudaSuccess) {
            c->sceneArena.release();
            return cuda_fail(c, x, "cudaMemcpy(scene)");
        }
    const tr_status bst = upload_bvh(c, wide);
    if (bst != TR_OK) {
        c->sceneArena.release();
        return bst;
    }
    const auto t2 = std::chrono::steady_clock::now();

    SceneView& s = c->scene;
    s.tris = reinterpret_cast<const TriShade*>(b + oTris);
    s.matIdx = reinterpret_cast<const uint32_t*>(b + oMat);
    s.materials = reinterpret_cast<const Material*>(b + oMats);
    s.lights = reinterpret_cast<const LightTri*>(b + oLights);
    s.alias = reinterpret_cast<const AliasEntry*>(b + oAlias);
    s.invTransforms = reinterpret_cast<const float4*>(b + oXf);
    s.texSlots = fs.texSlots.empty() ? nullptr : reinterpret_cast<const TexSlots*>(b + oTex);
    c->texSlotsHost = fs.texSlots;
    TR_CUDA(c, cudaMemset(b + oBins, 0, 2 * size_t(desc->material_count) * sizeof(uint32_t)));
    c->sort.counts = reinterpret_cast<uint32_t*>(b + oBins);
    c->sort.cursor = c->sort.counts + desc->material_count;
    c->sort.bins = desc->material_count;
    s.lightCount = int32_t(fs.lights.size());
    s.lightEnergy = fs.lightEnergy;
    s.lightEnergyTotal = fs.lightEnergyTotal;
    s.triCount = triCount;

    tr_scene_info& in = c->info;
    in = tr_scene_info{};
    in.triangle_count = triCount;
    in.light_count = uint32_t(fs.lights.size());
    in.material_count = desc->material_count;
    in.bvh_node_count = uint32_t(wide.nodes.size() + wide.tlasNodes.size());
    in.device_bytes = off + c->bvhArena.bytes;
    in.light_energy = fs.lightEnergyTotal;
    in.build_time_ms = std::chrono::duration<float, std::milli>(t1 - t0).count();
    in.upload_time_ms = std::chrono::duration<float, std::milli>(t2 - t1).count();
    for (int i = 0; i < 6; ++i)
        in.scene_bounds[i] = fs.bounds[i];
    c->hostLights = fs.lights;
    c->hostMatIdx = fs.matIdx;
    c->geom.assign(*desc);
    c->meshTriBase = fs.meshTriBase;
    c->leafSize = opt.maxLeafSize;
    c->tuning.bvh_leaf_size = opt.maxLeafSize;
    c->materialCount = desc->material_count;
    c->hasScene = true;
    c->sampleCount = 0;
    if (c->frame.sampleCount)
        cudaMemset(c->frame.sampleCount, 0, sizeof(uint32_t));
    return TR_OK;
}

tr_status tr_update_materials(void* ctx, const tr_material_desc* materials, uint32_t count)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (!c->hasScene)
        return fail(c, TR_ERR_NO_SCENE, "no scene uploaded");
    if (!materials || count != c->materialCount)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "material count differs from the uploaded scene");
    for (uint32_t i = 0; i < count; ++i)
        if (materials[i].closure > TR_CLOSURE_DISNEY)
            return fail(c, TR_ERR_INVALID_ARGUMENT, "unknown closure");
    // the emissive triangles must stay the same set: only their radiance may change
    size_t emissiveTris = 0;
    for (uint32_t m : c->hostMatIdx) {
        const tr_material_desc& d = materials[m];
        if (d.emissive[0] + d.emissive[1] + d.emissive[2] > kEpsilon)
            ++emissiveTris;
    }
    if (emissiveTris != c->hostLights.size())
        return fail(c, TR_ERR_INVALID_ARGUMENT, "the set of emissive triangles changed: upload the scene again");
    std::vector<Material> mats(count);
    for (uint32_t i = 0; i < count; ++i)
        mats[i] = resolve_material(materials[i]);
    // the textures stay assigned; the textured resolution reads the new emissive colour
    std::vector<TexSlots> slots = c->texSlotsHost;
    for (uint32_t i = 0; i < count && !slots.empty(); ++i) {
        for (uint32_t p = 0; p < TR_PROP_COUNT; ++p)
            if (slots[i].tex[p])
                mats[i].texMask |= 1u << p;
        for (int k = 0; k < 3; ++k)
            slots[i].emissive[k] = round_to_half(materials[i].emissive[k]);
    }
    std::vector<LightTri> lights = c->hostLights;
    std::vector<double> energies(lights.size());
    float sumEnergy = 0.f;
    for (size_t i = 0; i < lights.size(); ++i) {
        LightTri& lt = lights[i];
        const tr_material_desc& d = materials[c->hostMatIdx[size_t(lt.triIx)]];
        if (!(d.emissive[0] + d.emissive[1] + d.emissive[2] > kEpsilon))
            return fail(c, TR_ERR_INVALID_ARGUMENT, "the set of emissive triangles changed: upload the scene again");
        lt.radiance = make_float3(d.emissive[0], d.emissive[1], d.emissive[2]);
        const float3 e = lt.radiance * lt.area;
        lt.energy = e.x + e.y + e.z;
        lt.sumEnergy = sumEnergy;
        sumEnergy += lt.energy;
        energies[i] = double(lt.energy);
    }
    const std::vector<AliasEntry> alias = build_alias_table(energies);
    cudaSetDevice(c->device);
    if (c->stream)
        TR_CUDA(c, cudaStreamSynchronize(c->stream));
    TR_CUDA(c, cudaMemcpy(const_cast<Material*>(c->scene.materials), mats.data(), mats.size() * sizeof(Material),
                          cudaMemcpyHostToDevice));
    if (!slots.empty()) {
        TR_CUDA(c, cudaMemcpy(const_cast<TexSlots*>(c->scene.texSlots), slots.data(), slots.size() * sizeof(TexSlots),
                              cudaMemcpyHostToDevice));
        c->texSlotsHost = slots;
    }
    if (!lights.empty()) {
        TR_CUDA(c, cudaMemcpy(const_cast<LightTri*>(c->scene.lights), lights.data(), lights.size() * sizeof(LightTri),
                              cudaMemcpyHostToDevice));
        TR_CUDA(c, cudaMemcpy(const_cast<AliasEntry*>(c->scene.alias), alias.data(), alias.size() * sizeof(AliasEntry),
                              cudaMemcpyHostToDevice));
    }
    c->hostLights = lights;
    c->scene.lightEnergy = lights.empty() ? 0.f : lights.back().sumEnergy;
    c->scene.lightEnergyTotal = sumEnergy;
    c->info.light_energy = sumEnergy;
    invalidate_graph(c);  // light energies are kernel parameters
    return tr_reset(ctx);
}

tr_status tr_adjoint_frame(void* ctx, void* stream, const float* pixel_grad, float scale, float* param_grad)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (!pixel_grad || !param_grad)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "null gradient buffer");
    if (c->settings.flags & TR_FLAG_REFERENCE_SAMPLING)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "the adjoint differentiates the default sampling mode only");
    if (c->scene.sky.enabled)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "the adjoint differentiates scenes without a sky");
    if (c->scene.texSlots)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "the adjoint differentiates untextured materials only");
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    if (c->sampleCount < c->settings.multiSample)
        return fail(c, TR_ERR_NOT_READY, "render a frame before its adjoint");
    cudaSetDevice(c->device);
    const size_t cap = c->frame.capacity;
    if (!c->adjointArena.base) {
        // lrem 16 B + pending 32 B + NEE payload 32 B + visible slot 4 B per path, and the counters
        size_t off = 0;
        auto take = [&](size_t bytes) {
            const size_t o = off;
            off = align256(off + bytes);
            return o;
        };
        const size_t oL = take(cap * sizeof(float4));
        const size_t oP = take(2 * cap * sizeof(float4));
        const size_t oS = take(2 * cap * sizeof(float4));
        const size_t oV = take(cap * sizeof(uint32_t));
        const size_t oC = take(kCounterWords * sizeof(uint32_t));
        void* base = nullptr;
        const cudaError_t e = cudaMalloc(&base, off);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "cudaMalloc(adjoint scratch)");
        c->adjointArena.base = base;
        c->adjointArena.bytes = off;
        char* b = static_cast<char*>(base);
        c->adjoint.lrem = reinterpret_cast<float4*>(b + oL);
        c->adjoint.pending = reinterpret_cast<float4*>(b + oP);
        c->adjoint.shadowAdj = reinterpret_cast<float4*>(b + oS);
        c->adjoint.visible = reinterpret_cast<uint32_t*>(b + oV);
        c->adjointCounters = reinterpret_cast<uint32_t*>(b + oC);
    }
    AdjointView a = c->adjoint;
    a.pixelGrad = reinterpret_cast<const float4*>(pixel_grad);
    a.grads = param_grad;
    a.scale = scale;
    a.materialCount = c->materialCount;
    a.sampleBase = c->sampleCount - c->settings.multiSample;
    // the replay keeps the forward frame's statistics: its queues are reused, its counters are its own
    FrameView f = c->frame;
    f.counters = c->adjointCounters;
    TR_CUDA(c, launch_adjoint(c->scene, f, c->camera, c->settings, a, c->shape, pick_stream(c, stream)));
    return TR_OK;
}

tr_status tr_set_render_mode(void* ctx, uint32_t mode, uint32_t flags, float ao_dist, float z_depth_max)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (mode > kModeZDepth)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "unknown render mode");
    if (!(ao_dist > 0.f) || !(z_depth_max > 0.f))
        return fail(c, TR_ERR_INVALID_ARGUMENT, "ao_dist and z_depth_max must be > 0");
    const bool changed = mode != c->renderMode || flags != c->renderFlags || ao_dist != c->aoDist ||
                         z_depth_max != c->zDepthMax;
    c->renderMode = mode;
    c->renderFlags = flags;
    c->aoDist = ao_dist;
    c->zDepthMax = z_depth_max;
    if (changed) {
        invalidate_graph(c);
        return tr_reset(ctx);
    }
    return TR_OK;
}

tr_status tr_set_sky(void* ctx, const tr_sky_desc* sky)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (sky) {
        const float* d = sky->sun_dir;
        if (!std::isfinite(d[0]) || !std::isfinite(d[1]) || !std::isfinite(d[2]) ||
            !(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] > 0.f))
            return fail(c, TR_ERR_INVALID_ARGUMENT, "sun_dir must be a finite non-zero vector");
        if (!std::isfinite(sky->sun_angular_diameter) || !std::isfinite(sky->sun_intensity) ||
            !std::isfinite(sky->turbidity) || !std::isfinite(sky->selection_bias))
            return fail(c, TR_ERR_INVALID_ARGUMENT, "sky parameters must be finite");
        c->scene.sky = make_sky(*sky);
    } else {
        c->scene.sky = SkyView{};
    }
    invalidate_graph(c);
    return tr_reset(ctx);
}

tr_status tr_pick_ray(void* ctx, void* stream, int32_t x, int32_t y, tr_ray_pick_result* out)
{
    if (!ctx || !out)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    cudaSetDevice(c->device);
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    cudaStream_t s = pick_stream(c, stream);
    TR_CUDA(c, launch_pick_ray(c->scene, c->camera, c->settings, c->width, c->height, x, y, c->pickResult,
                               c->frame.errorFlag, s));
    float r[9];
    TR_CUDA(c, cudaMemcpyAsync(r, c->pickResult, sizeof(r), cudaMemcpyDeviceToHost, s));
    TR_CUDA(c, cudaStreamSynchronize(s));
    static_assert(sizeof(tr_ray_pick_result) == sizeof(r), "tr_ray_pick_result is 9 words");
    std::memcpy(out, r, sizeof(r));
    return TR_OK;
}

tr_status tr_get_tuning(void* ctx, tr_tuning* out)
{
    if (!ctx || !out)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    tr_tuning t = c->tuning;
    t.bvh_leaf_size = c->leafSize;
    t.bvh_nodes = c->hasScene ? (c->scene.quantNodes ? 2u : 1u) : c->nodeMode;
    if (c->shape.sms) {
        t.refill_below = c->shape.refillBelow;
        t.extend_blocks_per_sm = c->shape.extendBlocks / c->shape.sms;
        t.connect_blocks_per_sm = c->shape.connectBlocks / c->shape.sms;
        t.shade_waves = c->shape.shadeWaves;
        t.sort_hits = c->shape.sortHits;
        t.traversal_threads = c->shape.traversalThreads;
        t.shade_threads = c->shape.shadeThreads;
    }
    *out = t;
    return TR_OK;
}

tr_status tr_set_tuning(void* ctx, const tr_tuning* t)
{
    if (!ctx || !t)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    auto threadsOk = [](uint32_t v) { return v == 0 || v == 64 || v == 128; };
    if (t->bvh_leaf_size > 3 || t->refill_below > 32 || t->shade_waves > 64 || t->sort_hits > 1 ||
        !threadsOk(t->traversal_threads) || !threadsOk(t->shade_threads) || t->bvh_nodes > 2)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "tuning out of range (leaf size <= 3, refill <= 32, shade waves <= 64, "
                                                "block sizes 64 or 128, node layout <= 2)");
    cudaSetDevice(c->device);
    if (c->hasScene) {
        const tr_status st = rebuild_bvh(c, t->bvh_leaf_size ? t->bvh_leaf_size : c->leafSize, t->bvh_nodes);
        if (st != TR_OK)
            return st;
    } else {
        c->nodeMode = t->bvh_nodes;
    }
    c->tuning = *t;
    c->tuning.bvh_leaf_size = c->leafSize;
    invalidate_graph(c);
    if (c->frameArena.base) {
        c->shape = tuned_launch_shape(c->device, uint32_t(c->frame.capacity), c->tuning);
        c->frame.hitOrder = c->shape.sortHits ? c->sort.order : nullptr;
    }
    return TR_OK;
}

// Coordinate search over the tunables, each configuration timed over two
// graph-replayed frames after one warm-up frame.
tr_status tr_autotune(void* ctx, void* stream, uint32_t flags, tr_tune_report* report)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    cudaSetDevice(c->device);
    st = ensure_frame(c);
    if (st != TR_OK)
        return st;
    cudaStream_t s = pick_stream(c, stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TR_CUDA(c, cudaEventCreate(&e0));
    TR_CUDA(c, cudaEventCreate(&e1));
    uint32_t trials = 0;
    const bool samples = (flags & TR_TUNE_SAMPLES) != 0;
    const uint32_t spp = 4u * c->settings.multiSample;
    auto timeFrames = [&](float* ms) -> tr_status {
        const int timed = samples ? 1 : 2;
        auto render = [&]() { return samples ? tr_render_samples(ctx, stream, spp, 1) : tr_render_frame(ctx, stream, 1); };
        tr_status r = render();
        if (r != TR_OK)
            return r;
        TR_CUDA(c, cudaEventRecord(e0, s));
        for (int i = 0; i < timed && r == TR_OK; ++i)
            r = render();
        if (r != TR_OK)
            return r;
        TR_CUDA(c, cudaEventRecord(e1, s));
        TR_CUDA(c, cudaEventSynchronize(e1));
        TR_CUDA(c, cudaEventElapsedTime(ms, e0, e1));
        *ms /= float(timed);
        ++trials;
        return TR_OK;
    };
    tr_tuning best{};
    tr_get_tuning(ctx, &best);
    float bestMs = 0.f, defaultMs = 0.f;
    st = timeFrames(&bestMs);
    defaultMs = bestMs;
    auto tryTuning = [&](const tr_tuning& t) -> tr_status {
        tr_status r = tr_set_tuning(ctx, &t);
        if (r != TR_OK)
            return r;
        float ms = 0.f;
        r = timeFrames(&ms);
        if (r != TR_OK)
            return r;
        if (ms < bestMs) {
            bestMs = ms;
            best = t;
        }
        return TR_OK;
    };
    // block sizes first: the grids below are counted in blocks of the chosen size
    for (uint32_t v : {64u}) {
        tr_tuning t = best;
        t.traversal_threads = v;
        t.extend_blocks_per_sm = 0;
        t.connect_blocks_per_sm = 0;
        if (st == TR_OK && v != best.traversal_threads)
            st = tryTuning(t);
    }
    for (uint32_t v : {64u}) {
        tr_tuning t = best;
        t.shade_threads = v;
        if (st == TR_OK && v != best.shade_threads)
            st = tryTuning(t);
    }
    const uint32_t refills[] = {6, 8, 10, 12, 16, 20, 24, 28, 32};
    for (uint32_t v : refills) {
        tr_tuning t = best;
        t.refill_below = v;
        if (st == TR_OK && v != best.refill_below)
            st = tryTuning(t);
    }
    tr_tuning sized = best;
    sized.extend_blocks_per_sm = 0;
    sized.connect_blocks_per_sm = 0;
    const LaunchShape def = tuned_launch_shape(c->device, uint32_t(c->frame.capacity), sized);
    for (uint32_t d : {def.extendPerSm / 2, def.extendPerSm * 3 / 4}) {
        tr_tuning t = best;
        t.extend_blocks_per_sm = d;
        if (st == TR_OK && d >= 1 && d != best.extend_blocks_per_sm)
            st = tryTuning(t);
    }
    for (uint32_t d : {def.connectPerSm / 2, def.connectPerSm * 3 / 4}) {
        tr_tuning t = best;
        t.connect_blocks_per_sm = d;
        if (st == TR_OK && d >= 1 && d != best.connect_blocks_per_sm)
            st = tryTuning(t);
    }
    for (uint32_t w : {1u, 2u, 8u}) {
        tr_tuning t = best;
        t.shade_waves = w;
        if (st == TR_OK && w != best.shade_waves)
            st = tryTuning(t);
    }
    if (!samples) {
        tr_tuning t = best;
        t.sort_hits = best.sort_hits ? 0u : 1u;
        if (st == TR_OK)
            st = tryTuning(t);
    }
    if ((flags & TR_TUNE_SKIP_BVH) == 0) {
        for (uint32_t leaf : {1u, 2u, 3u}) {
            tr_tuning t = best;
            t.bvh_leaf_size = leaf;
            if (st == TR_OK && leaf != best.bvh_leaf_size)
                st = tryTuning(t);
        }
        // the other node layout (fp32 or quantized child boxes)
        tr_tuning t = best;
        t.bvh_nodes = c->scene.quantNodes ? 1u : 2u;
        if (st == TR_OK)
            st = tryTuning(t);
    }
    if (st == TR_OK)
        st = tr_set_tuning(ctx, &best);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != TR_OK)
        return st;
    tr_reset(ctx);
    if (report) {
        *report = tr_tune_report{};
        tr_get_tuning(ctx, &report->chosen);
        report->frame_ms_default = defaultMs;
        report->frame_ms_tuned = bestMs;
        report->trials = trials;
    }
    return TR_OK;
}

tr_status tr_get_scene_info(void* ctx, tr_scene_info* info)
{
    if (!ctx || !info)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (!c->hasScene)
        return fail(c, TR_ERR_NO_SCENE, "no scene uploaded");
    *info = c->info;
    return TR_OK;
}

tr_status tr_set_camera(void* ctx, const tr_camera* cam)
{
    if (!ctx || !cam)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    Camera k{};
    std::string err;
    if (!convert_camera(*cam, &k, &err))
        return fail(c, TR_ERR_INVALID_ARGUMENT, err);
    if (c->hasCamera && std::memcmp(&k, &c->camera, sizeof(Camera)) == 0)
        return TR_OK;  // unchanged camera: keep the accumulation and the captured frame graph
    c->camera = k;
    c->hasCamera = true;
    invalidate_graph(c);
    return tr_reset(ctx);
}

tr_status tr_set_settings(void* ctx, const tr_kernel_settings* s)
{
    if (!ctx || !s)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (s->multi_sample == 0)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "multi_sample must be >= 1 and max_depth in [1, 16]");
    Settings k{};
    std::string err;
    if (!convert_settings(*s, &k, &err))
        return fail(c, TR_ERR_INVALID_ARGUMENT, err);
    const bool changed = std::memcmp(&k, &c->settings, sizeof(Settings)) != 0;
    c->settings = k;
    if (changed) {
        invalidate_graph(c);
        return tr_reset(ctx);
    }
    return TR_OK;
}

tr_status tr_resize(void* ctx, uint32_t width, uint32_t height)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (width == 0 || height == 0 || uint64_t(width) * height >= TR_MAX_PATHS)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "resolution must be non-zero with width*height < 2^28");
    c->width = width;
    c->height = height;
    return tr_reset(ctx);
}

tr_status tr_reset(void* ctx)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    c->sampleCount = 0;
    if (c->frame.sampleCount && c->frameArena.base) {
        cudaSetDevice(c->device);
        TR_CUDA(c, cudaMemsetAsync(c->frame.sampleCount, 0, sizeof(uint32_t), c->stream));
        TR_CUDA(c, cudaMemsetAsync(c->frame.traversal, 0, kTraversalCounters * sizeof(unsigned long long), c->stream));
        TR_CUDA(c, cudaMemsetAsync(c->frame.errorFlag, 0, sizeof(uint32_t), c->stream));
        TR_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return TR_OK;
}

tr_status tr_begin_frame(void* ctx, void* stream)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    cudaSetDevice(c->device);
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    c->timedFrame = false;
    c->lastFrameNoalloc = false;
    c->lastSamples = false;
    c->lastStream = pick_stream(c, stream);
    return enqueue_begin(c, c->lastStream);
}

tr_status tr_generate(void* ctx, void* stream)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    TR_CUDA(c, launch_generate(c->frame, c->camera, c->settings, pick_stream(c, stream)));
    return TR_OK;
}

tr_status tr_extend(void* ctx, void* stream, uint32_t bounce)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (bounce >= TR_MAX_DEPTH)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "bounce out of range");
    if (c->renderMode != kModePathTracing)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "the stage entries drive the path-tracing mode; render other modes "
                                                "with tr_render_frame");
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    TR_CUDA(c, launch_extend(c->scene, c->frame, c->settings, bounce, c->shape, pick_stream(c, stream)));
    if (c->shape.sortHits)
        TR_CUDA(c, launch_sort_hits(c->scene, c->frame, c->sort, bounce, c->shape, pick_stream(c, stream)));
    return TR_OK;
}

tr_status tr_shade(void* ctx, void* stream, uint32_t bounce)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (bounce >= TR_MAX_DEPTH)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "bounce out of range");
    if (c->renderMode != kModePathTracing)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "the stage entries drive the path-tracing mode; render other modes "
                                                "with tr_render_frame");
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    TR_CUDA(c, launch_shade(c->scene, c->frame, c->settings, bounce, c->shape, pick_stream(c, stream)));
    return TR_OK;
}

tr_status tr_connect(void* ctx, void* stream, uint32_t bounce)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if (bounce >= TR_MAX_DEPTH)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "bounce out of range");
    if (c->renderMode != kModePathTracing)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "the stage entries drive the path-tracing mode; render other modes "
                                                "with tr_render_frame");
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    TR_CUDA(c, launch_connect(c->scene, c->frame, c->settings, bounce, c->shape, pick_stream(c, stream)));
    return TR_OK;
}

tr_status tr_finalize(void* ctx, void* stream)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    TR_CUDA(c, launch_finalize(c->frame, c->settings, pick_stream(c, stream)));
    c->sampleCount += c->settings.multiSample;
    return TR_OK;
}

tr_status tr_render_frame(void* ctx, void* stream, int32_t use_graph)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    cudaSetDevice(c->device);
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    cudaStream_t s = pick_stream(c, stream);
    c->lastStream = s;
    c->lastFrameNoalloc = false;
    c->lastSamples = false;
    if (use_graph) {
        if (!c->graphValid) {
            // capture on the context stream (the legacy default stream cannot be captured)
            TR_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            st = enqueue_frame(c, c->stream, false);
            cudaGraph_t g = nullptr;
            const cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
            if (st != TR_OK) {
                if (g)
                    cudaGraphDestroy(g);
                return st;
            }
            if (ec != cudaSuccess)
                return cuda_fail(c, ec, "cudaStreamEndCapture");
            c->graph = g;
            TR_CUDA(c, cudaGraphInstantiate(&c->graphExec, g, 0));
            c->graphValid = true;
        }
        TR_CUDA(c, cudaGraphLaunch(c->graphExec, s));
        c->timedFrame = false;
    } else {
        st = enqueue_frame(c, s, true);
        if (st != TR_OK)
            return st;
        c->timedFrame = true;
        c->timedDepth = c->settings.maxDepth;
    }
    c->sampleCount += c->settings.multiSample;
    return TR_OK;
}

// tr_render_samples: one continuous wavefront of width * height * spp samples
// through the frame's path slots (the batch kernels with one item), or, where
// those kernels do not apply, spp / multi_sample frames.
tr_status tr_render_samples(void* ctx, void* stream, uint32_t spp, int32_t use_graph)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    cudaSetDevice(c->device);
    tr_status st = check_ready(c);
    if (st != TR_OK)
        return st;
    const uint32_t ms = c->settings.multiSample;
    if (spp == 0 || spp % ms != 0)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "spp must be a positive multiple of multi_sample");
    const uint64_t wh = uint64_t(c->width) * c->height;
    const uint64_t samples = wh * spp;
    const uint32_t flags = c->settings.flags;
    const bool continuous = c->renderMode == kModePathTracing &&
                            (flags & (TR_FLAG_REFERENCE_SAMPLING | TR_FLAG_WRITE_AOVS)) == 0 && samples <= (1ull << 30);
    if (!continuous) {
        for (uint32_t k = 0; k < spp / ms && st == TR_OK; ++k)
            st = tr_render_frame(ctx, stream, use_graph);
        return st;
    }
    // per-sample radiance, the item and the iteration state
    if (c->samplesCapacity < samples) {
        invalidate_graph(c);
        c->samplesArena.release();
        c->samplesCapacity = 0;
        const size_t oRad = 0;
        const size_t oItem = align256(size_t(samples) * sizeof(float4));
        const size_t oState = align256(oItem + sizeof(BatchItem));
        const size_t bytes = align256(oState + sizeof(BatchState));
        void* base = nullptr;
        const cudaError_t e = cudaMalloc(&base, bytes);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "cudaMalloc(sample radiance)");
        c->samplesArena.base = base;
        c->samplesArena.bytes = bytes;
        char* b = static_cast<char*>(base);
        c->sampleRadiance = reinterpret_cast<float4*>(b + oRad);
        c->samplesItem = reinterpret_cast<BatchItem*>(b + oItem);
        c->samplesState = reinterpret_cast<BatchState*>(b + oState);
        c->samplesCapacity = samples;
    }
    BatchItem it{};
    it.camera = c->camera;
    it.width = c->width;
    it.height = c->height;
    it.root = 0;
    it.lightBase = 0;
    it.lightCount = c->scene.lightCount;
    it.lightEnergy = c->scene.lightEnergy;
    it.lightEnergyTotal = c->scene.lightEnergyTotal;
    it.pixelBase = 0;
    it.spp = spp;
    it.sampleBase = 0;
    cudaStream_t s = pick_stream(c, stream);
    if (!c->samplesItemValid || std::memcmp(&it, &c->samplesItemHost, sizeof(BatchItem)) != 0) {
        c->samplesItemHost = it;
        TR_CUDA(c, cudaMemcpy(c->samplesItem, &c->samplesItemHost, sizeof(BatchItem), cudaMemcpyHostToDevice));
        c->samplesItemValid = true;
    }
    FrameView f = c->frame;
    f.radiance = c->sampleRadiance;
    f.batch = c->samplesState;
    f.items = c->samplesItem;
    f.itemCount = 1;
    f.hitOrder = nullptr;
    f.pathCount = uint32_t(c->frameCapacity);
    LaunchShape shape = c->shape;
    shape.sortHits = 0;
    const ContinuousLaunch L{c->scene, c->settings, shape, uint32_t(c->frameCapacity), c->side, c->evFork,
                             c->evJoin};
    const std::vector<ContinuousRound> rounds{ContinuousRound{f, uint32_t(samples), 0u, uint32_t(wh)}};
    if (use_graph && (flags & TR_FLAG_COUNT_TRAVERSAL) == 0) {
        if (!c->samplesExec || c->samplesGraphSpp != spp) {
            if (c->samplesExec)
                cudaGraphExecDestroy(c->samplesExec);
            if (c->samplesGraph)
                cudaGraphDestroy(c->samplesGraph);
            c->samplesExec = nullptr;
            c->samplesGraph = nullptr;
            // captured on the context's own stream, which must be idle
            TR_CUDA(c, cudaStreamSynchronize(c->stream));
            cudaGraph_t g = nullptr;
            TR_CUDA(c, capture_continuous(L, rounds, spp, c->stream, &g));
            c->samplesGraph = g;
            TR_CUDA(c, cudaGraphInstantiate(&c->samplesExec, g, 0));
            c->samplesGraphSpp = spp;
        }
        TR_CUDA(c, cudaGraphLaunch(c->samplesExec, s));
        c->samplesTimed = false;
    } else {
        // eager: stage by stage with a host loop, each stage timed by CUDA events
        c->samplesTimes = StageTimes{};
        c->samplesTimed = false;
        TR_CUDA(c, run_continuous_eager(L, rounds, spp, s, &c->samplesTimes));
        c->samplesTimed = true;
    }
    c->lastStream = s;
    c->timedFrame = false;
    c->lastFrameNoalloc = false;
    c->lastSamples = true;
    c->lastSamplesPaths = uint32_t(samples);
    c->sampleCount += spp;
    return TR_OK;
}

tr_status tr_synchronize(void* ctx, void* stream)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    cudaSetDevice(c->device);
    TR_CUDA(c, cudaStreamSynchronize(pick_stream(c, stream)));
    return TR_OK;
}

tr_status tr_get_statistics(void* ctx, tr_statistics* out)
{
    if (!ctx || !out)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    FrameWords words{c->frame.counters, c->frame.sampleCount, c->frame.errorFlag, c->frame.traversal};
    uint32_t primary = c->frame.pathCount;
    if (c->lastFrameNoalloc) {
        // the last frame came from tr_render_frame_noalloc: its words live in the shared scratch
        std::string err;
        const tr_status st = noalloc_frame_words(c->device, &words, err);
        if (st != TR_OK)
            return fail(c, st, err);
        primary = c->noallocPaths;
    } else if (!c->frameArena.base) {
        return fail(c, TR_ERR_NOT_READY, "no frame rendered");
    }
    cudaSetDevice(c->device);
    TR_CUDA(c, cudaDeviceSynchronize());
    uint32_t counters[kCounterWords];
    TR_CUDA(c, cudaMemcpy(counters, words.counters, sizeof(counters), cudaMemcpyDeviceToHost));
    uint32_t err = 0, sc = 0;
    unsigned long long trav[kTraversalCounters] = {};
    TR_CUDA(c, cudaMemcpy(trav, words.traversal, sizeof(trav), cudaMemcpyDeviceToHost));
    TR_CUDA(c, cudaMemcpy(&err, words.errorFlag, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    TR_CUDA(c, cudaMemcpy(&sc, words.sampleCount, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    tr_statistics s{};
    if (c->lastSamples) {
        // the continuous wavefront keeps totals, not per-bounce queue lengths
        BatchState bs{};
        TR_CUDA(c, cudaMemcpy(&bs, c->samplesState, sizeof(bs), cudaMemcpyDeviceToHost));
        s.primary_path_count = c->lastSamplesPaths;
        s.secondary_path_count = bs.extendRays - c->lastSamplesPaths;
        s.shadow_ray_count = bs.shadowRays;
        s.path_count = bs.extendRays + bs.shadowRays;
        s.sample_count = sc;
        s.device_error = err;
        s.traversal_extend_nodes = trav[0];
        s.traversal_extend_tris = trav[1];
        s.traversal_connect_nodes = trav[2];
        s.traversal_connect_tris = trav[3];
        s.radiance_updates_shade = trav[4];
        s.radiance_updates_connect = trav[5];
        s.hit_ray_count = bs.hitRays;
        s.iterations = bs.iterations;
        // kernels: finalize, advance, and plan + connect + extend + shade per iteration (the
        // last finds nothing to trace); the round-start memset is not a kernel
        s.launches = 2u + 4u * (bs.iterations + 1u);
        if (c->samplesTimed) {
            const StageTimes& t = c->samplesTimes;
            s.generate_time_ms = t.plan;
            s.extend_time_ms = t.extend;
            s.shade_time_ms = t.shade;
            s.connect_time_ms = t.connect;
            s.finalize_time_ms = t.end;
            s.render_time_ms = t.plan + t.extend + t.shade + t.connect + t.end;
        }
        *out = s;
        return TR_OK;
    }
    const uint32_t depth = c->settings.maxDepth;
    for (uint32_t b = 0; b < depth; ++b) {
        s.extend_rays[b] = b == 0 ? primary : counters[b];
        s.shadow_rays[b] = counters[kShadowCounterBase + b];
        s.hit_rays[b] = counters[kHitCounterBase + b];
        s.path_count += s.extend_rays[b] + s.shadow_rays[b];
        s.shadow_ray_count += s.shadow_rays[b];
        s.hit_ray_count += s.hit_rays[b];
        if (b == 0)
            s.primary_path_count = s.extend_rays[b];
        else if (b == 1)
            s.secondary_path_count = s.extend_rays[b];
        else
            s.deep_path_count += s.extend_rays[b];
    }
    if (c->timedFrame) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->evStart, c->evFinal);
        s.render_time_ms = ms;
        cudaEventElapsedTime(&ms, c->evStart, c->evGenerate);
        s.generate_time_ms = ms;
        cudaEvent_t prev = c->evGenerate;
        for (uint32_t b = 0; b < c->timedDepth; ++b) {
            cudaEventElapsedTime(&ms, prev, c->evExtend[b]);
            s.extend_time_ms += ms;
            cudaEventElapsedTime(&ms, c->evExtend[b], c->evShade[b]);
            s.shade_time_ms += ms;
            cudaEventElapsedTime(&ms, c->evShade[b], c->evConnect[b]);
            s.connect_time_ms += ms;
            prev = c->evConnect[b];
        }
        cudaEventElapsedTime(&ms, prev, c->evFinal);
        s.finalize_time_ms = ms;
    }
    s.sample_count = sc;
    s.device_error = err;
    s.traversal_extend_nodes = trav[0];
    s.traversal_extend_tris = trav[1];
    s.traversal_connect_nodes = trav[2];
    s.traversal_connect_tris = trav[3];
    s.radiance_updates_shade = trav[4];
    s.radiance_updates_connect = trav[5];
    *out = s;
    return TR_OK;
}

tr_status tr_get_buffers(void* ctx, tr_buffers* out)
{
    if (!ctx || !out)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    tr_status st = ensure_frame(c);
    if (st != TR_OK)
        return st;
    tr_buffers b{};
    b.path_state[0] = c->frame.state[0];
    b.path_state[1] = c->frame.state[1];
    b.hits = c->frame.hits;
    b.shadow = c->frame.shadow;
    b.radiance = c->frame.radiance;
    b.accumulator = c->frame.accumulator;
    b.albedo = c->frame.albedo;
    b.normals = c->frame.normals;
    b.colors = c->frame.colors;
    b.counters = c->frame.counters;
    b.capacity = c->frame.capacity;
    b.width = c->frame.resX;
    b.height = c->frame.resY;
    *out = b;
    return TR_OK;
}

static tr_status download(Context* c, void* stream, const void* src, float* dst, uint64_t bytes)
{
    if (!c->frameArena.base)
        return fail(c, TR_ERR_NOT_READY, "no frame rendered");
    const uint64_t need = uint64_t(c->frame.resX) * c->frame.resY * sizeof(float4);
    if (!dst || bytes < need)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "destination smaller than width*height*16 bytes");
    cudaSetDevice(c->device);
    cudaStream_t s = pick_stream(c, stream);
    TR_CUDA(c, cudaMemcpyAsync(dst, src, need, cudaMemcpyDeviceToHost, s));
    TR_CUDA(c, cudaStreamSynchronize(s));
    return TR_OK;
}

tr_status tr_download_image(void* ctx, void* stream, float* host_rgba, uint64_t bytes)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    return download(c, stream, c->frame.colors, host_rgba, bytes);
}

tr_status tr_download_accumulator(void* ctx, void* stream, float* host_rgba, uint64_t bytes)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    return download(c, stream, c->frame.accumulator, host_rgba, bytes);
}

tr_status tr_copy_from_device(void* ctx, void* host_dst, const void* device_src, uint64_t bytes)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if ((!host_dst || !device_src) && bytes)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "null pointer");
    cudaSetDevice(c->device);
    TR_CUDA(c, cudaDeviceSynchronize());
    TR_CUDA(c, cudaMemcpy(host_dst, device_src, bytes, cudaMemcpyDeviceToHost));
    return TR_OK;
}

tr_status tr_copy_to_device(void* ctx, void* device_dst, const void* host_src, uint64_t bytes)
{
    if (!ctx)
        return TR_ERR_INVALID_ARGUMENT;
    Context* c = static_cast<Context*>(ctx);
    if ((!device_dst || !host_src) && bytes)
        return fail(c, TR_ERR_INVALID_ARGUMENT, "null pointer");
    cudaSetDevice(c->device);
    TR_CUDA(c, cudaDeviceSynchronize());
    TR_CUDA(c, cudaMemcpy(device_dst, host_src, bytes, cudaMemcpyHostToDevice));
    return TR_OK;
}

} // extern "C"
