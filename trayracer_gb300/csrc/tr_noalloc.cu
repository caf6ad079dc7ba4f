// One wavefront frame into caller-owned buffers without allocating device
// memory (tr_render_frame_noalloc).
//
// Some callers cannot allocate device memory where they render: a real-time
// loop that must not stall the device (cudaMalloc and cudaFree synchronise it),
// a host application that hands out all device memory from its own pool or
// budget, or code running where no allocating call is permitted. For them the
// frame's scratch - the two path-state queues, the hit and shadow queues, the
// per-path radiance and the queue counters - lives in one file-scope device
// array of fixed size instead of the context's frame buffers. The array is part
// of the library's device image: every GPU that loads the library holds it
// (about 22 MiB) until the process exits.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/trayracer.h"
#include "tr_api_internal.h"
#include "tr_kernels.h"

namespace tr {
namespace {

// Paths in flight (width * height * multi_sample) one call can hold.
constexpr uint32_t kNoAllocMaxPaths = 1u << 17;
// Per path: two 3-plane state queues (96 B), hit (16 B), 3-plane shadow queue (48 B), radiance (16 B).
constexpr size_t kNoAllocPathBytes = 2 * 3 * 16 + 16 + 3 * 16 + 16;
constexpr size_t kNoAllocTailBytes = 1024;  // counters, sample count, error word, traversal counters
constexpr size_t kNoAllocScratchBytes = size_t(kNoAllocMaxPaths) * kNoAllocPathBytes + kNoAllocTailBytes;
static_assert(kCounterWords * 4 + 4 + 4 <= 512 && 512 + kTraversalCounters * 8 <= kNoAllocTailBytes,
              "scratch tail too small");

__device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setupMutex;
void* g_scratchAddress[kMaxDevices] = {};

// Makes `device` current for the guard's lifetime and restores the calling
// thread's previous device afterwards.
struct DeviceGuard {
    int previous = -1;
    bool ok = false;
    explicit DeviceGuard(int device)
    {
        if (cudaGetDevice(&previous) != cudaSuccess)
            previous = -1;
        ok = previous == device || cudaSetDevice(device) == cudaSuccess;
    }
    ~DeviceGuard()
    {
        if (previous >= 0)
            cudaSetDevice(previous);
    }
};

// Clears what a frame expects to start at zero and sets the frame's sample count.
__global__ void noalloc_begin_kernel(uint32_t* counters, uint32_t* sampleCount, uint32_t* errorFlag,
                                     unsigned long long* traversal, uint32_t sc)
{
    for (uint32_t i = threadIdx.x; i < kCounterWords; i += blockDim.x)
        counters[i] = 0u;
    if (threadIdx.x == 0) {
        *sampleCount = sc;
        *errorFlag = 0u;
        for (uint32_t k = 0; k < kTraversalCounters; ++k)
            traversal[k] = 0ull;
    }
}

// Device address of the scratch array on `device` (current). Looked up once per
// device; the lookup loads the library's device image on that device if it was
// not loaded yet.
tr_status scratch_address(int device, void** out, std::string& err)
{
    if (device < 0 || device >= kMaxDevices) {
        err = "device ordinal out of range for the no-allocation scratch table";
        return TR_ERR_LIMIT;
    }
    std::lock_guard<std::mutex> lock(g_setupMutex);
    if (!g_scratchAddress[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess || !p) {
            err = std::string("cudaGetSymbolAddress(no-allocation scratch): ") + cudaGetErrorString(e);
            return TR_ERR_CUDA;
        }
        g_scratchAddress[device] = p;
    }
    *out = g_scratchAddress[device];
    return TR_OK;
}

// Where the frame's buffers sit in the scratch array at `base` for `cap` paths.
FrameView scratch_frame(char* base, size_t cap)
{
    FrameView f{};
    f.state[0] = reinterpret_cast<float4*>(base);
    f.state[1] = reinterpret_cast<float4*>(base + 3 * cap * 16);
    f.hits = reinterpret_cast<uint4*>(base + 6 * cap * 16);
    f.shadow = reinterpret_cast<float4*>(base + 7 * cap * 16);
    f.radiance = reinterpret_cast<float4*>(base + 10 * cap * 16);
    char* tail = base + size_t(kNoAllocMaxPaths) * kNoAllocPathBytes;
    f.counters = reinterpret_cast<uint32_t*>(tail);
    f.sampleCount = reinterpret_cast<uint32_t*>(tail + kCounterWords * 4);
    f.errorFlag = reinterpret_cast<uint32_t*>(tail + kCounterWords * 4 + 4);
    f.traversal = reinterpret_cast<unsigned long long*>(tail + 512);
    f.capacity = uint32_t(cap);
    return f;
}

} // namespace

tr_status noalloc_frame_words(int device, FrameWords* out, std::string& err)
{
    DeviceGuard guard(device);
    if (!guard.ok) {
        err = "cudaSetDevice failed";
        return TR_ERR_CUDA;
    }
    void* base = nullptr;
    const tr_status st = scratch_address(device, &base, err);
    if (st != TR_OK)
        return st;
    const FrameView f = scratch_frame(static_cast<char*>(base), 0);
    *out = FrameWords{f.counters, f.sampleCount, f.errorFlag, f.traversal};
    return TR_OK;
}

} // namespace tr

using namespace tr;

extern "C" tr_status tr_render_frame_noalloc(void* ctx, void* stream, float* accumulator, float* colors,
                                             uint32_t sample_count)
{
    ContextViews v;
    tr_status st = context_views(ctx, &v);
    if (st != TR_OK)
        return st;
    if (!accumulator || !colors)
        return context_fail(ctx, TR_ERR_INVALID_ARGUMENT, "accumulator and colors must be device pointers");
    if (v.renderMode != kModePathTracing)
        return context_fail(ctx, TR_ERR_INVALID_ARGUMENT,
                            "tr_render_frame_noalloc renders the path-tracing mode only; render other modes "
                            "with tr_render_frame");
    const uint64_t wh = uint64_t(v.width) * v.height;
    const uint64_t paths = wh * v.settings.multiSample;
    if (paths == 0 || paths > kNoAllocMaxPaths)
        return context_fail(ctx, TR_ERR_LIMIT,
                            "tr_render_frame_noalloc holds at most 131072 paths in flight "
                            "(width * height * multi_sample)");
    DeviceGuard guard(v.device);
    if (!guard.ok)
        return context_fail(ctx, TR_ERR_CUDA, "cudaSetDevice failed");
    void* base = nullptr;
    std::string err;
    st = scratch_address(v.device, &base, err);
    if (st != TR_OK)
        return context_fail(ctx, st, err);

    const size_t cap = size_t(paths);
    FrameView f = scratch_frame(static_cast<char*>(base), cap);
    f.accumulator = reinterpret_cast<float4*>(accumulator);
    f.colors = reinterpret_cast<float4*>(colors);
    f.albedo = nullptr;
    f.normals = nullptr;
    f.resX = v.width;
    f.resY = v.height;
    f.pathCount = uint32_t(paths);
    f.hitOrder = nullptr;

    Settings s = v.settings;
    s.flags &= ~uint32_t(TR_FLAG_WRITE_AOVS);  // no guide buffers on this path
    LaunchShape shape;
    st = context_launch_shape(ctx, uint32_t(cap), &shape);
    if (st != TR_OK)
        return st;
    cudaStream_t cs = stream ? static_cast<cudaStream_t>(stream) : v.stream;

    noalloc_begin_kernel<<<1, 128, 0, cs>>>(f.counters, f.sampleCount, f.errorFlag, f.traversal, sample_count);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = launch_generate(f, v.camera, s, cs);
    for (uint32_t bounce = 0; e == cudaSuccess && bounce < s.maxDepth; ++bounce) {
        e = launch_extend(v.scene, f, s, bounce, shape, cs);
        if (e == cudaSuccess)
            e = launch_shade(v.scene, f, s, bounce, shape, cs);
        if (e == cudaSuccess)
            e = launch_connect(v.scene, f, s, bounce, shape, cs);
    }
    if (e == cudaSuccess)
        e = launch_finalize(f, s, cs);
    if (e != cudaSuccess)
        return context_fail(ctx, TR_ERR_CUDA, std::string("tr_render_frame_noalloc: ") + cudaGetErrorString(e));
    context_note_noalloc_frame(ctx, uint32_t(paths));
    return TR_OK;
}
