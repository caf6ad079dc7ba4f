// Wavefront path-tracing kernels for sm_103a: generate, extend, shade,
// connect, finalize.
//
// Data layout (all in HBM):
//   path state  3 float4 planes per queue (coalesced 16-byte accesses): the
//               extend queue (rays of the bounce) and the hit queue (the rays
//               that hit something, state copied by the extend launch next to
//               their hit record); extend reads the first and fills the
//               second, shade reads the second and refills the first, so no
//               launch reads and writes the same queue (the reference
//               compacts in place, PathTracing.h:16-18 vs :171-173) and
//               missed rays (black sky) never reach the shade launch;
//   hits        one uint4 per hit-queue slot;
//   shadow      3 float4 planes, compacted;
//   radiance    one float4 per path index; every contribution of a path is
//               added here by the only thread that owns the path in that
//               stage, so no atomics are needed and the per-pixel sum in
//               finalize runs in a fixed sample order (the reference adds into
//               the pixel with plain read-modify-writes from many paths,
//               PathTracing.h:45,90 and optix.cu:340).
// Queue appends use one warp ballot + one atomicAdd per warp.
#include "tr_kernels.h"
#include "tr_sky.h"

#include <type_traits>

#include "tr_bsdf.cuh"
#include "tr_bsdf_dual.cuh"
#include "tr_rng.h"
#include "tr_traverse.cuh"

#include <cuda_fp16.h>

namespace tr {

namespace {

constexpr uint32_t kFull = 0xffffffffu;

__device__ __forceinline__ float h2f(uint16_t h) { return __half2float(__ushort_as_half(h)); }

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// 16-byte asynchronous global -> shared copy (L2 only), its commit and the wait
// for all of this thread's committed copies.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Appends the lanes with pred set to a queue; one atomic per warp.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred)
{
    const uint32_t mask = __ballot_sync(kFull, pred);
    if (mask == 0)
        return 0;
    const uint32_t lane = lane_id();
    const uint32_t leader = __ffs(mask) - 1u;
    uint32_t base = 0;
    if (lane == leader)
        base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(kFull, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// Two appends at once (one atomic per warp and queue, both in flight before
// either result is read): slot0 / slot1 of the lanes with pred0 / pred1.
__device__ __forceinline__ void warp_append2(uint32_t* counter0, bool pred0, uint32_t& slot0, uint32_t* counter1,
                                             bool pred1, uint32_t& slot1)
{
    const uint32_t m0 = __ballot_sync(kFull, pred0);
    const uint32_t m1 = __ballot_sync(kFull, pred1);
    const uint32_t lane = lane_id();
    const uint32_t l0 = m0 ? __ffs(m0) - 1u : 0u;
    const uint32_t l1 = m1 ? __ffs(m1) - 1u : 0u;
    uint32_t b0 = 0, b1 = 0;
    if (m0 && lane == l0)
        b0 = atomicAdd(counter0, __popc(m0));
    if (m1 && lane == l1)
        b1 = atomicAdd(counter1, __popc(m1));
    b0 = __shfl_sync(kFull, b0, l0);
    b1 = __shfl_sync(kFull, b1, l1);
    const uint32_t below = (1u << lane) - 1u;
    slot0 = b0 + __popc(m0 & below);
    slot1 = b1 + __popc(m1 & below);
}

// SafeColor = fixnan(clamp_scaled(c, max)), CudaUtility.h:95-99 and
// CudaLinearMath.h:127-142.
__device__ __forceinline__ float3 safe_color(const float3& c, float maxValue)
{
    float3 r = c;
    const float m = fmaxf(c.x, fmaxf(c.y, c.z));
    if (!(m <= maxValue))
        r = c * (maxValue / m);
    return isfinite(r.x + r.y + r.z) ? r : f3(0.f);
}

__device__ __forceinline__ float3 fixnan(const float3& c) { return isfinite(c.x + c.y + c.z) ? c : f3(0.f); }

__device__ __forceinline__ uint32_t encode_bary(float u, float v)
{
    const uint32_t bx = static_cast<uint32_t>(u * 65535.f) & 0xFFFFu;
    const uint32_t by = static_cast<uint32_t>(v * 65535.f) & 0xFFFFu;
    return (bx << 16) | by;
}

__device__ __forceinline__ float2 decode_bary(uint32_t b)
{
    return make_float2(static_cast<float>(b >> 16) / 65535.f, static_cast<float>(b & 0xFFFFu) / 65535.f);
}

// PackNormal as stored by the reference (CudaUtility.h:153-160: the x and y
// components, saturated to 16 bits); kept for the D.w payload only.
__device__ __forceinline__ uint32_t pack_normal(const float3& n)
{
    return (__float2uint_rz(n.x * 65535.f) << 16) | __float2uint_rz(n.y * 65535.f);
}

// ------------------------------------------------------------------ camera
// Two draws in argument order: left to right, or right to left when rtl.
template <class Rng>
__device__ __forceinline__ void draw2(Rng& rng, bool rtl, float& a, float& b)
{
    if (rtl) {
        b = rng.next();
        a = rng.next();
    } else {
        a = rng.next();
        b = rng.next();
    }
}

template <class Rng>
__device__ __forceinline__ float2 sample_disk(Rng& rng, bool rtl)
{
    float ux, uy;
    draw2(rng, rtl, ux, uy);
    const float lx = (ux * 2.f) - 1.f;
    const float ly = (uy * 2.f) - 1.f;
    if (lx == 0 && ly == 0)
        return make_float2(lx, ly);
    float theta, r;
    if (fabsf(lx) > fabsf(ly)) {
        r = lx;
        theta = kPiOver4 * (ly / lx);
    } else {
        r = ly;
        theta = kPiOver2 - kPiOver4 * (lx / ly);
    }
    float s, c;
    sincosf(theta, &s, &c);
    return make_float2(r * c, r * s);
}

template <class Rng>
__device__ __forceinline__ float2 sample_bokeh(const Camera& cam, Rng& rng, bool rtl)
{
    if (cam.bokehSideCount < 3)
        return sample_disk(rng, rtl);
    const int index = static_cast<int>(rng.next() * cam.bokehSideCount);
    const float step = (2.f * kPi) / cam.bokehSideCount;
    float s0, c0, s1, c1;
    sincosf(cam.bokehRotation + (index * step), &s0, &c0);
    sincosf(cam.bokehRotation + (index + 1) * step, &s1, &c1);
    const float u1 = rng.next();
    const float u2 = rng.next();
    const float su = sqrtf(u1);
    // SampleTriangle(c0 = 0, c1, c2), optix.cu:82-88
    return (su * (1 - u2)) * make_float2(c0, s0) + (su * u2) * make_float2(c1, s1);
}

__device__ __forceinline__ bool distort(float2& lens, float tanFov2, float distortion)
{
    if (lens.x == 0 && lens.y == 0)
        return true;
    if (distortion <= 0)
        return true;
    const float scale = sqrtf(lens.x * lens.x + lens.y * lens.y);
    const float d = (tanFov2 * distortion) * .5f;
    const float distorted = (scale * distortion * atanf(d)) / d;
    if (distorted >= kPiOver2)
        return false;
    lens = lens * (tanf(distorted) / (scale * distortion));
    return true;
}

// GenerateCameraRay, optix.cu:142-174
template <class Rng>
__device__ __forceinline__ void camera_ray(const Camera& cam, uint32_t resX, uint32_t resY, int ix, int iy,
                                           Rng& rng, bool rtl, float3& O, float3& D, float& T)
{
    O = cam.pos;
    D = cam.forward;
    T = 1.f;
    float jx, jy;
    draw2(rng, rtl, jx, jy);
    const float rx = float(resX), ry = float(resY);
    const float aspect = rx / ry;
    float2 screen = make_float2((((float(ix) + jx) / rx) * 2.0f) - 1.f, (((float(iy) + jy) / ry) * 2.0f) - 1.f);
    screen.y /= aspect;
    const float2 ccd = sample_bokeh(cam, rng, rtl) * cam.aperture;
    float2 lens = make_float2((cam.tanFov2 * screen.x) - (ccd.x / cam.focalDist),
                              (cam.tanFov2 * screen.y) - (ccd.y / cam.focalDist));
    if (!distort(lens, cam.tanFov2, cam.distortion))
        return;
    D = normalize(cam.forward + (lens.x * cam.side) + (lens.y * cam.up));
    O = cam.pos + (cam.side * ccd.x) + (cam.up * ccd.y);
    const float v = fmaxf(0.f, dot(D, cam.forward));
    const float v2 = v * v;
    T = v2 * v2;
}

// Batched rendering: the item of a sample id (items sorted by sampleBase).
__device__ __forceinline__ uint32_t batch_item(const FrameView& f, uint32_t id)
{
    uint32_t lo = 0, hi = f.itemCount;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&f.items[mid].sampleBase) <= id)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// Item, pixel and sample index of a batch sample id.
struct BatchSample {
    uint32_t item;
    uint32_t pixel;
    uint32_t sample;
};
__device__ __forceinline__ BatchSample batch_sample(const FrameView& f, uint32_t id)
{
    BatchSample b;
    b.item = batch_item(f, id);
    const uint32_t local = id - __ldg(&f.items[b.item].sampleBase);
    const uint32_t spp = __ldg(&f.items[b.item].spp);
    b.pixel = local / spp;
    b.sample = local - b.pixel * spp;
    return b;
}

// Per-path item, bounce and flags of a batched path, kept in D.w (the packed
// normal of one-scene paths, which nothing reads): item << 8 | bounce << 4 |
// flags, so that no stage searches the items for a path's sample id again.
constexpr uint32_t kBatchItemShift = 8;
__device__ __forceinline__ uint32_t batch_pack(uint32_t bounce, uint32_t flags, uint32_t item)
{
    return (item << kBatchItemShift) | ((bounce & 0xfu) << kPathIxShift) | (flags & kFlagsMask);
}
__device__ __forceinline__ uint32_t batch_bounce(uint32_t packed) { return (packed >> kPathIxShift) & 0xfu; }
__device__ __forceinline__ uint32_t batch_item_of(uint32_t packed) { return packed >> kBatchItemShift; }

// Pixel and sample index of a batch sample id of a known item.
__device__ __forceinline__ BatchSample batch_sample_in(const FrameView& f, uint32_t id, uint32_t item)
{
    BatchSample b;
    b.item = item;
    const uint32_t local = id - __ldg(&f.items[item].sampleBase);
    const uint32_t spp = __ldg(&f.items[item].spp);
    b.pixel = local / spp;
    b.sample = local - b.pixel * spp;
    return b;
}

// BVH root of a batch item.
__device__ __forceinline__ uint32_t item_root(const FrameView& f, uint32_t item) { return __ldg(&f.items[item].root); }

// The scene view of a batch item: the concatenated buffers with the item's
// light range.
__device__ __forceinline__ SceneView item_scene(const SceneView& s, const BatchItem& it)
{
    SceneView si = s;
    si.lights = s.lights + it.lightBase;
    si.alias = s.alias + it.lightBase;
    si.lightCount = it.lightCount;
    si.lightEnergy = it.lightEnergy;
    si.lightEnergyTotal = it.lightEnergyTotal;
    return si;
}

// ------------------------------------------------------------------ kernels
// Primary ray of a path (the camera half of the Primary raygen program,
// optix.cu:235-276): sc = samples accumulated before this frame.
template <bool REF, bool BATCH>
__device__ __forceinline__ void primary_ray(const FrameView& f, const Camera& cam, const Settings& st, uint32_t pathIx,
                                            uint32_t sc, float3& O, float3& D, float& T, uint32_t* itemOut = nullptr)
{
    const uint32_t wh = f.resX * f.resY;
    const uint32_t pixelIx = pathIx % wh;
    const uint32_t sampleIx = pathIx / wh;
    if (BATCH) {
        // pathIx is the sample id: the item's camera and film, the counter RNG
        // keyed as for one scene
        // itemOut (optional) comes in as an item at or before the sample's and
        // goes out as the sample's item
        BatchSample bs;
        if (itemOut) {
            uint32_t item = *itemOut;
            while (item + 1u < f.itemCount && __ldg(&f.items[item + 1u].sampleBase) <= pathIx)
                ++item;
            *itemOut = item;
            bs = batch_sample_in(f, pathIx, item);
        } else {
            bs = batch_sample(f, pathIx);
        }
        const BatchItem& it = f.items[bs.item];
        CounterRng rng;
        rng.init(bs.pixel, sc + bs.sample, 0u, st.seed);
        camera_ray(it.camera, it.width, it.height, bs.pixel % it.width, bs.pixel / it.width, rng, false, O, D, T);
    } else if (REF) {
        RefRng rng{tea2(st.seed + pathIx, sc << 1)};
        const bool rtl = (st.flags & TR_FLAG_REFERENCE_DRAW_RTL) != 0;
        camera_ray(cam, f.resX, f.resY, pixelIx % f.resX, pixelIx / f.resX, rng, rtl, O, D, T);
    } else {
        CounterRng rng;
        rng.init(pixelIx, sc + sampleIx, 0u, st.seed);
        camera_ray(cam, f.resX, f.resY, pixelIx % f.resX, pixelIx / f.resX, rng, false, O, D, T);
    }
}

// Work item i of a launch that makes its camera rays -> the path it traces: the
// samples of a pixel are consecutive, and the pixels are taken in 8 x 4 tiles,
// so that a warp starts the nearly identical camera rays of one or two pixels
// (its 32 lanes hold 32 / multi_sample pixels) and the rest of the frame keeps
// that coherence: their hits, shadow rays and bounce rays sit together in the
// queues. A permutation of [0, W*H*ms); a film that is not a whole number of
// tiles takes its pixels row by row. The order in which paths are traced changes
// no path's result (radiance and random numbers are keyed by the path index).
__device__ __forceinline__ uint32_t camera_order(const FrameView& f, uint32_t i)
{
    const uint32_t W = f.resX, H = f.resY;
    const uint32_t wh = W * H;
    const uint32_t ms = f.pathCount / wh;
    const uint32_t sample = i % ms, r = i / ms;
    if ((W & 7u) || (H & 3u))
        return sample * wh + r;
    const uint32_t tile = r >> 5, within = r & 31u;
    const uint32_t tilesX = W >> 3;
    const uint32_t ty = tile / tilesX, tx = tile - ty * tilesX;
    return sample * wh + ((ty << 2) | (within >> 3)) * W + ((tx << 3) | (within & 7u));
}

template <bool REF, bool BATCH>
__global__ void __launch_bounds__(256) generate_kernel(FrameView f, Camera cam, Settings st)
{
    const uint32_t pathIx = blockIdx.x * blockDim.x + threadIdx.x;
    if (pathIx >= f.pathCount)
        return;
    float3 O, D;
    float T;
    primary_ray<REF, BATCH>(f, cam, st, pathIx, *f.sampleCount, O, D, T);
    const uint32_t cap = f.capacity;
    float4* s = f.state[0];
    s[pathIx] = f4(O, u2f(pack_path(pathIx, 0)));
    s[pathIx + cap] = f4(D, 0.f);
    s[pathIx + 2 * cap] = make_float4(T, T, T, 1.f);
    f.radiance[pathIx] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ uint32_t queue_length(const FrameView& f, uint32_t bounce)
{
    return bounce == 0 ? f.pathCount : __ldcg(f.counters + bounce);
}

// Sums per-thread traversal work into a device counter, one atomic per warp.
// Adds the warp's sum of v to *dst (one atomic per warp).
__device__ __forceinline__ void add_count(unsigned long long* dst, uint32_t v)
{
    unsigned long long n = v;
    for (int o = 16; o > 0; o >>= 1)
        n += __shfl_down_sync(kFull, n, o);
    if (lane_id() == 0 && n)
        atomicAdd(dst, n);
}

__device__ __forceinline__ void add_counts(unsigned long long* dst, const TraversalCounts& c)
{
    unsigned long long n = c.nodes, t = c.tris;
    for (int o = 16; o > 0; o >>= 1) {
        n += __shfl_down_sync(kFull, n, o);
        t += __shfl_down_sync(kFull, t, o);
    }
    if (lane_id() == 0) {
        atomicAdd(dst, n);
        atomicAdd(dst + 1, t);
    }
}

// Persistent warps refill a lane with the next ray of the queue when fewer
// than st.refillBelow of its 32 rays are still traversing (incoherent
// secondary rays end at very different times); tuned per scene, 10 by default
// (what the autotuner picks on the benchmark heightfield, 8 to 10).
constexpr uint32_t kRefillBelow = 10;

// Closest hit of the bounce's extend queue. Rays that hit are appended (one
// warp ballot and one atomic per step) to the hit queue with their full path
// state and hit record; missed rays end here. COUNT = true also sums the nodes
// visited and triangles tested (for the traversal bytes of the roofline); it
// is launched outside timed regions. PRIMARY = true (bounce 0 of a frame
// rendered as a whole, default sampling mode) computes each path's camera ray
// in place of reading a generated queue, and clears the path's radiance: the
// primary rays never go through memory.
// A path that leaves the scene sees the sky (PathTracing.h:40-55): T * SampleSky,
// with the sun disc for camera and specular paths; a primary miss writes the sky
// as its albedo guide. Out of line so that the traversal loop keeps its registers.
// BATCH: the path's sample id is O.w, its bounce and flags are in D.w.
template <bool BATCH>
__device__ __noinline__ void sky_miss(const SceneView& s, const FrameView& f, const Settings& st, uint32_t bounce,
                                      float4 O4, float4 D4, float4 T4, bool aov)
{
    const uint32_t data = __float_as_uint(O4.w);
    const uint32_t pathIx = BATCH ? data : path_ix(data);
    const uint32_t flags = BATCH ? (__float_as_uint(D4.w) & kFlagsMask) : path_flags(data);
    if (BATCH)
        bounce = batch_bounce(__float_as_uint(D4.w));
    const bool sun = s.sky.drawSun != 0.f && (bounce == 0 || (flags & kFlagSpecular));
    const float3 sky = sky_radiance(s.sky, f3(D4), sun);
    const float3 add = safe_color(f3(T4) * sky, st.maxColor);
    const float4 r = f.radiance[pathIx];
    f.radiance[pathIx] = make_float4(r.x + add.x, r.y + add.y, r.z + add.z, r.w);
    if (aov && pathIx < f.resX * f.resY) {
        f.albedo[pathIx] = f4(sky, 0.f);
        f.normals[pathIx] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// BATCH: the extend queue of a batch iteration - entries [0, carried) are
// paths carried over from the last iteration, the entries after them start
// new samples (their camera rays are made here), so the pool stays full.
// Blocks of 64 or 128 threads (a launch parameter, LaunchShape::traversalThreads):
// the kernel works per warp; 64 registers, 32 resident warps per SM.
template <bool COUNT, bool BATCH, bool PRIMARY, bool TL, int LAYOUT = kLayoutScene>
__global__ void __launch_bounds__(128, 8) extend_kernel(SceneView s, FrameView f, Settings st, uint32_t bounce,
                                                     Camera cam)
{
    const uint32_t count = BATCH ? __ldcg(&f.batch->queue) : queue_length(f, bounce);
    const uint32_t carried = BATCH ? __ldcg(&f.batch->carried) : 0u;
    const uint32_t freshBase = BATCH ? __ldcg(&f.batch->freshBase) : 0u;
    const float4* __restrict__ in = f.state[0];
    float4* __restrict__ hq = f.state[1];
    const uint32_t cap = f.capacity;
    uint32_t* work = BATCH ? &f.batch->extendWork : f.counters + kExtendWorkBase + bounce;
    uint32_t* hitCounter = BATCH ? &f.batch->hits : f.counters + kHitCounterBase + bounce;
    const uint32_t lane = lane_id();
    const bool aov = (st.flags & TR_FLAG_WRITE_AOVS) && bounce == 0;
    const uint32_t wh = f.resX * f.resY;
    TraversalCounts cnt{0, 0};
    typename TravOf<TL>::type t;
    uint2 stack[kTraversalStack];
    float4 O4 = make_float4(0.f, 0.f, 0.f, 0.f), D4 = O4, T4 = O4;
    const uint32_t sc = (PRIMARY || BATCH) ? *f.sampleCount : 0u;
    bool alive = false, more = true;
    while (true) {
        const uint32_t idle = __ballot_sync(kFull, !alive && more);
        if (idle) {
            const uint32_t leader = __ffs(idle) - 1u;
            uint32_t first = 0;
            if (lane == leader)
                first = atomicAdd(work, __popc(idle));
            first = __shfl_sync(kFull, first, leader);
            // batched: the item of the first new sample of this refill, found by the
            // whole warp (the first sample ids of 32 items per load and a ballot, in
            // place of a binary search per lane); the refill's new sample ids are
            // consecutive, so a lane's own item is at most a few further
            uint32_t warpItem = 0;
            if (BATCH && f.itemCount > 1u && first + __popc(idle) > carried && first < count) {
                const uint32_t firstFresh = freshBase + (first > carried ? first - carried : 0u);
                for (uint32_t j0 = 1u; j0 < f.itemCount; j0 += 32u) {
                    const uint32_t j = j0 + lane;
                    const uint32_t m =
                        __ballot_sync(kFull, j < f.itemCount && __ldg(&f.items[j].sampleBase) <= firstFresh);
                    warpItem += __popc(m);
                    if (m != kFull)
                        break;  // items are in sample order: none later starts at or before it
                }
            }
            if (!alive && more) {
                const uint32_t i = first + __popc(idle & ((1u << lane) - 1u));
                if (i < count) {
                    if (BATCH ? i >= carried : PRIMARY) {
                        float3 O, D;
                        float T;
                        uint32_t item = warpItem;
                        const uint32_t pathIx = BATCH ? freshBase + (i - carried) : camera_order(f, i);
                        primary_ray<false, BATCH>(f, cam, st, pathIx, sc, O, D, T, &item);
                        // a batch path keeps its sample id in O.w and item | bounce | flags in D.w
                        O4 = f4(O, u2f(BATCH ? pathIx : pack_path(pathIx, 0)));
                        D4 = f4(D, BATCH ? u2f(batch_pack(0u, 0u, item)) : 0.f);
                        T4 = make_float4(T, T, T, 1.f);
                        f.radiance[pathIx] = make_float4(0.f, 0.f, 0.f, 0.f);
                    } else {
                        O4 = __ldcs(in + i);
                        D4 = __ldcs(in + i + cap);
                        T4 = __ldcs(in + i + 2 * cap);
                    }
                    traversal_begin(t, f3(O4), f3(D4), st.rayEpsilon, kDstMax,
                                    BATCH ? item_root(f, batch_item_of(__float_as_uint(D4.w))) : 0u);
                    alive = true;
                } else {
                    more = false;
                }
            }
        }
        if (!__any_sync(kFull, alive))
            break;
        uint32_t active;
        do {
            bool done = false;
            if (alive)
                done = traversal_step<false, COUNT, LAYOUT>(t, stack, s, &cnt);
            const bool hit = done && base(t).hitSlot != 0xffffffffu;
            const uint32_t slot = warp_append(hitCounter, hit);
            if (done) {
                if (!base(t).ok)
                    atomicOr(f.errorFlag, 1u);
                if (hit) {
                    const uint32_t prim = __float_as_uint(__ldg(s.bvhTris + 3u * base(t).hitSlot).w);
                    __stcs(hq + slot, O4);
                    __stcs(hq + slot + cap, D4);
                    __stcs(hq + slot + 2 * cap, T4);
                    __stcs(f.hits + slot, make_uint4(encode_bary(base(t).u, base(t).v), hit_instance(t), prim,
                                                     __float_as_uint(base(t).tmax)));
                } else if (s.sky.enabled) {
                    sky_miss<BATCH>(s, f, st, bounce, O4, D4, T4, aov);
                } else if (aov) {
                    // a primary miss sees the disabled sky: black guide values (PathTracing.h:48-52)
                    const uint32_t pathIx = path_ix(__float_as_uint(O4.w));
                    if (pathIx < wh) {
                        f.albedo[pathIx] = make_float4(0.f, 0.f, 0.f, 0.f);
                        f.normals[pathIx] = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                }
                alive = false;
            }
            active = __ballot_sync(kFull, alive);
        } while (uint32_t(__popc(active)) >= st.refillBelow);
    }
    if (COUNT)
        add_counts(f.traversal, cnt);
}

// Light sample, CudaLights.h:38-124.
template <bool REF, class Rng>
__device__ __forceinline__ float3 sample_light(const SceneView& s, Rng& rng, bool rtl, const float3& I,
                                               const float3& N, float& prob, float& pdf, float3& radiance,
                                               float& dist, int32_t& lightOut)
{
    lightOut = -1;
    const float total = REF ? s.lightEnergy : s.lightEnergyTotal;
    if (total == 0 || s.lightCount == 0) {
        prob = 0;
        pdf = 0;
        radiance = f3(0.f);
        dist = 1e20f;
        return make_float3(0, 1, 0);
    }
    int32_t lightIx;
    float3 P;
    if (REF) {
        // binary search over the exclusive energy prefix (SelectLight)
        const float e = rng.next() * s.lightEnergy;
        int32_t low = 0, high = s.lightCount - 1;
        lightIx = -1;
        for (int it = 0; it < 64 && low <= high; ++it) {
            const int32_t mid = (low + high) >> 1;
            const float se = __ldg(&s.lights[mid].sumEnergy);
            const float en = __ldg(&s.lights[mid].energy);
            if (e < se) {
                high = mid;
            } else if (e > se + en) {
                low = mid + 1;
            } else {
                lightIx = mid;
                break;
            }
        }
        if (lightIx < 0) {
            const int c = static_cast<int>(rng.next() * s.lightCount);
            lightIx = c < 0 ? 0 : (c > s.lightCount - 1 ? s.lightCount - 1 : c);
        }
        const LightTri& L = s.lights[lightIx];
        float b0, b1, b2;
        if (rtl) {
            b2 = rng.next();
            b1 = rng.next();
            b0 = rng.next();
        } else {
            b0 = rng.next();
            b1 = rng.next();
            b2 = rng.next();
        }
        P = (b0 * L.V0) + (b1 * L.V1) + (b2 * L.V2);
    } else {
        const float u = rng.next();
        const float coin = rng.next();
        uint32_t k = static_cast<uint32_t>(u * float(s.lightCount));
        k = k < uint32_t(s.lightCount) ? k : uint32_t(s.lightCount) - 1u;
        const AliasEntry a = s.alias[k];
        lightIx = int32_t(coin < a.prob ? k : a.alias);
        const LightTri& L = s.lights[lightIx];
        const float r0 = rng.next(), r1 = rng.next();
        const float su = sqrtf(r0);
        P = ((1.f - su) * L.V0) + ((su * (1.f - r1)) * L.V1) + ((su * r1) * L.V2);
    }
    lightOut = lightIx;
    const LightTri& L = s.lights[lightIx];
    float3 Ld = I - P;
    const float sqDist = dot(Ld, Ld);
    Ld = normalize(Ld);
    const float LNdotL = dot(L.N, Ld);
    prob = fdiv(L.energy, total);
    const bool facing = REF ? (dot(N, Ld) != 0.f) : (dot(N, Ld) < 0.f);
    pdf = (LNdotL > 0 && facing) ? fdiv(sqDist, L.area * LNdotL) : 0;
    dist = sqrtf(sqDist);
    radiance = L.radiance;
    return -Ld;
}

__device__ __forceinline__ float3 xform(const float4& tx, const float4& ty, const float4& tz, const float3& v)
{
    return make_float3(dot(v, make_float3(tx.x, ty.x, tz.x)), dot(v, make_float3(tx.y, ty.y, tz.y)),
                       dot(v, make_float3(tx.z, ty.z, tz.z)));
}

struct Surface {
    float3 N;   // shading normal
    float3 Ng;  // geometric normal
    float3 T;   // tangent
    float3 B;   // bitangent
    float area;
    uint32_t matIx;
    float2 uv;  // texture coordinate
};

// tex2D of a property's texture: its RGB (GetColor, CudaMaterial.h:89-92)
__device__ __forceinline__ float3 tex_rgb(unsigned long long t, const float2& uv)
{
    const float4 c = tex2D<float4>(t, uv.x, uv.y);
    return make_float3(c.x, c.y, c.z);
}

// GetIntersectionAttributes + FixNormals, CudaMaterial.h:117-212 (TEX: the scene has
// textures, so a normal map may apply)
template <bool TEX = false>
__device__ __forceinline__ Surface surface_at(const SceneView& s, uint32_t instIx, uint32_t primIx, float2 bary,
                                              const float3& D)
{
    Surface sf;
    // two-level scenes: primIx counts in the instance's mesh
    const uint32_t triIx = (s.instInfo ? __ldg(&s.instInfo[instIx].y) : 0u) + primIx;
    const TriShade& tri = s.tris[triIx];
    sf.matIx = __ldg(s.matIdx + triIx);
    const float3 v0 = make_float3(tri.v0x, tri.v0y, tri.v0z);
    const float3 v1 = make_float3(tri.v1x, tri.v1y, tri.v1z);
    const float3 v2 = make_float3(tri.v2x, tri.v2y, tri.v2z);
    const float3 e1 = v1 - v0;
    const float3 e2 = v2 - v0;
    sf.area = length(cross(e1, e2)) * 0.5f;
    const float3 N0 = make_float3(h2f(tri.N0x), h2f(tri.N0y), h2f(tri.N0z));
    const float3 N1 = make_float3(h2f(tri.N1x), h2f(tri.N1y), h2f(tri.N1z));
    const float3 N2 = make_float3(h2f(tri.N2x), h2f(tri.N2y), h2f(tri.N2z));
    sf.N = normalize(N0 + ((N1 - N0) * bary.x) + ((N2 - N0) * bary.y));
    sf.Ng = make_float3(h2f(tri.Nx), h2f(tri.Ny), h2f(tri.Nz));
    const float2 uv0 = make_float2(h2f(tri.uv0x), h2f(tri.uv0y));
    const float2 uv1 = make_float2(h2f(tri.uv1x), h2f(tri.uv1y));
    const float2 uv2 = make_float2(h2f(tri.uv2x), h2f(tri.uv2y));
    sf.uv = make_float2(uv0.x + ((uv1.x - uv0.x) * bary.x) + ((uv2.x - uv0.x) * bary.y),
                        uv0.y + ((uv1.y - uv0.y) * bary.x) + ((uv2.y - uv0.y) * bary.y));
    if (TEX && (__ldg(&s.materials[sf.matIx].texMask) & (1u << TR_PROP_NORMAL))) {
        // normal map (CudaMaterial.h:185-191), applied where the reference applies it: before
        // the tangent frame is computed, so with the zero tangent and bitangent of its
        // zero-initialised Intersection; the map can only keep or flip the normal
        const float3 nm = tex_rgb(__ldg(&s.texSlots[sf.matIx].tex[TR_PROP_NORMAL]), sf.uv);
        const float3 norMap = (nm * 2.f) - f3(1.f);
        const float3 zero = f3(0.f);
        sf.N = normalize(norMap.x * zero + norMap.y * zero + norMap.z * sf.N);
    }

    // tangents from texcoord derivatives (differences taken in fp16)
    const __half u0x = __ushort_as_half(tri.uv0x), u0y = __ushort_as_half(tri.uv0y);
    const float s1 = __half2float(__hsub(__ushort_as_half(tri.uv1x), u0x));
    const float t1 = __half2float(__hsub(__ushort_as_half(tri.uv1y), u0y));
    const float s2 = __half2float(__hsub(__ushort_as_half(tri.uv2x), u0x));
    const float t2 = __half2float(__hsub(__ushort_as_half(tri.uv2y), u0y));
    const float r = (s1 * t2) - (s2 * t1);
    if (fabsf(r) < 1e-6f) {
        sf.B = normalize(cross(sf.N, e1));
        sf.T = normalize(cross(sf.N, sf.B));
    } else {
        const float rr = fdiv(1.f, r);
        const float3 tv = ((s1 * e2) - (s2 * e1)) * rr;
        sf.B = normalize(tv - sf.N * dot(sf.N, tv));
        sf.T = normalize(cross(sf.N, sf.B));
    }
    if (s.instInfo) {
        // two-level scenes: the frame to world space by the inverse-transpose
        // instance transform (one mesh: the identity, skipped)
        const float4 tx = __ldg(s.invTransforms + instIx * 3 + 0);
        const float4 ty = __ldg(s.invTransforms + instIx * 3 + 1);
        const float4 tz = __ldg(s.invTransforms + instIx * 3 + 2);
        sf.N = normalize(xform(tx, ty, tz, sf.N));
        sf.Ng = normalize(xform(tx, ty, tz, sf.Ng));
        sf.B = normalize(xform(tx, ty, tz, sf.B));
        sf.T = normalize(xform(tx, ty, tz, sf.T));
    }
    if (dot(D, sf.N) > 0) {
        sf.Ng = -sf.Ng;
        sf.N = -sf.N;
        sf.T = -sf.T;
        sf.B = -sf.B;
    }
    return sf;
}

__device__ __forceinline__ HitMat load_material(const Material* __restrict__ mats, uint32_t ix, uint32_t& closure,
                                                uint32_t& emissiveFlag, uint32_t* texMask = nullptr)
{
    const float4* p = reinterpret_cast<const float4*>(mats + ix);
    const float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3), e = __ldg(p + 4);
    const uint4 g = __ldg(reinterpret_cast<const uint4*>(p + 5));
    HitMat m;
    m.diffuse = make_float3(a.x, a.y, a.z);
    m.metallic = a.w;
    m.emissive = make_float3(b.x, b.y, b.z);
    m.subsurface = b.w;
    m.tint = make_float3(c.x, c.y, c.z);
    m.specular = c.w;
    m.roughness = d.x;
    m.specularTint = d.y;
    m.anisotropic = d.z;
    m.sheen = d.w;
    m.sheenTint = e.x;
    m.clearcoat = e.y;
    m.clearcoatGloss = e.z;
    m.luminance = e.w;
    closure = g.x;
    emissiveFlag = g.y;
    if (texMask)
        *texMask = g.z;
    return m;
}

// GetIntersectionAttributes' material part (CudaMaterial.h:153-183) for a material
// with textures: each textured property is its colour times the texture's RGB at
// the hit, then emissive = Emissive * diffuse, tint and luminance from the
// textured diffuse, and the emissive test of PathTracing.h:73 per hit.
__device__ __forceinline__ void apply_textures(const SceneView& s, uint32_t matIx, uint32_t mask, float2 uv, HitMat& m,
                                            uint32_t& emissiveFlag)
{
    const TexSlots& t = s.texSlots[matIx];
    auto scalar = [&](uint32_t p, float& v) {
        if (mask & (1u << p))
            v = v * tex_rgb(__ldg(&t.tex[p]), uv).x;
    };
    if (mask & (1u << TR_PROP_DIFFUSE))
        m.diffuse = m.diffuse * tex_rgb(__ldg(&t.tex[TR_PROP_DIFFUSE]), uv);
    const float3 tintXYZ = linear_to_xyz(m.diffuse);
    scalar(TR_PROP_METALLIC, m.metallic);
    m.emissive = make_float3(__ldg(&t.emissive[0]), __ldg(&t.emissive[1]), __ldg(&t.emissive[2])) * m.diffuse;
    scalar(TR_PROP_SUBSURFACE, m.subsurface);
    m.tint = tintXYZ.y > 0 ? xyz_to_linear(tintXYZ * (1.f / tintXYZ.y)) : f3(1.f);
    scalar(TR_PROP_SPECULAR, m.specular);
    scalar(TR_PROP_ROUGHNESS, m.roughness);
    scalar(TR_PROP_SPECULAR_TINT, m.specularTint);
    scalar(TR_PROP_ANISOTROPIC, m.anisotropic);
    scalar(TR_PROP_SHEEN, m.sheen);
    scalar(TR_PROP_SHEEN_TINT, m.sheenTint);
    scalar(TR_PROP_CLEARCOAT, m.clearcoat);
    scalar(TR_PROP_CLEARCOAT_GLOSS, m.clearcoatGloss);
    m.luminance = tintXYZ.y;
    emissiveFlag = (m.emissive.x + m.emissive.y + m.emissive.z > kEpsilon) ? 1u : 0u;
}

// What the path-replay adjoint needs to know about one shaded vertex.
struct VertexInfo {
    bool hit;
    bool emissive;
    float3 emitted;       // radiance added at an emissive hit (after SafeColor)
    uint32_t matIx;
    uint32_t closure;
    HitMat mat;
    float3 wo;            // tangent space
    float3 wiLight;
    float3 wiExt;
    int32_t lightIx;
};

// One PathTracingKernel step (PathTracing.h:15-174) for one queue entry. With
// vi == nullptr (the shade kernel) it adds emitted radiance and writes the
// guide buffers; the adjoint replay passes vi and gets the vertex instead.
// Returns true when it added emitted radiance to the path's radiance. BATCH:
// the path's sample id is O.w, its bounce and flags are in D.w, and its last
// bounce (max_depth - 1) makes no extend ray.
template <bool REF, class Rng, bool TEX = false, bool BATCH = false>
__device__ __forceinline__ bool shade_path(const SceneView& s, const FrameView& f, const Settings& st, uint32_t bounce,
                                           uint32_t sc, const float4& O4, const float4& D4, const float4& T4,
                                           const uint4& hd, Rng& rng, bool& wantExt, float4 (&ext)[3],
                                           bool& wantShadow, float4 (&sh)[3], VertexInfo* vi = nullptr)
{
    const uint32_t wh = f.resX * f.resY;
    const float3 O = f3(O4), D = f3(D4), T = f3(T4);
    const uint32_t data = __float_as_uint(O4.w);
    const uint32_t pathIx = BATCH ? data : path_ix(data);
    uint32_t flags = BATCH ? (__float_as_uint(D4.w) & kFlagsMask) : path_flags(data);
    const float extendPdf = T4.w;
    const uint32_t pixelIx = pathIx % wh;
    const bool aov = !BATCH && vi == nullptr && (st.flags & TR_FLAG_WRITE_AOVS) && bounce == 0 && pathIx < wh;
    if (vi) {
        vi->hit = false;
        vi->emissive = false;
        vi->lightIx = -1;
    }

    const float2 bary = decode_bary(hd.x);
    const uint32_t instIx = hd.y, primIx = hd.z;
    const float tmax = __uint_as_float(hd.w);
    const float3 I = O + D * tmax;

    if (primIx == 0xffffffffu) {
        // miss: only the adjoint replay comes here (the extend kernel shades misses, sky_miss),
        // and it takes scenes without a sky, where SampleSky returns black (CudaSky.h:108-109)
        if (aov) {
            f.albedo[pixelIx] = make_float4(0.f, 0.f, 0.f, 0.f);
            f.normals[pixelIx] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        return false;
    }

    const Surface sf = surface_at<TEX>(s, instIx, primIx, bary, D);
    uint32_t closure, emissiveFlag, texMask;
    HitMat m = load_material(s.materials, sf.matIx, closure, emissiveFlag, &texMask);
    if (TEX && texMask)
        apply_textures(s, sf.matIx, texMask, sf.uv, m, emissiveFlag);
    if (vi) {
        vi->hit = true;
        vi->matIx = sf.matIx;
        vi->closure = closure;
        vi->mat = m;
    }
    if (aov) {
        f.albedo[pixelIx] = f4(m.diffuse, 0.f);
        f.normals[pixelIx] = f4(sf.N, 0.f);
    }

    if (emissiveFlag) {
        float3 contrib = f3(0.f);
        if (bounce == 0 || (flags & kFlagSpecular)) {
            contrib = m.emissive;
        } else {
            const float lightPdf = fdiv(tmax * tmax, fabsf(dot(D, sf.N)) * sf.area);
            const float3 en = m.emissive * sf.area;
            const float total = REF ? s.lightEnergy : s.lightEnergyTotal;
            const float pick = fdiv(en.x + en.y + en.z, total);
            const float denom = extendPdf + lightPdf * pick;
            if (REF) {
                if (denom > 0)
                    contrib = T * m.diffuse * fdiv(1.0f, denom);
            } else {
                if (denom > 0)
                    contrib = T * m.emissive * fdiv(extendPdf, denom);
            }
        }
        float3 add = safe_color(contrib, st.maxColor);
        if (REF && bounce == 0)
            add += m.emissive;  // the reference adds the primary emission a second time (PathTracing.h:93-97)
        if (vi) {
            vi->emissive = true;
            vi->emitted = add;
            return false;
        }
        float4 r = f.radiance[pathIx];
        f.radiance[pathIx] = make_float4(r.x + add.x, r.y + add.y, r.z + add.z, r.w);
        return true;
    }

    float lightProb, lightPdf, lightDist;
    float3 lightRadiance;
    const bool rtl = REF && (st.flags & TR_FLAG_REFERENCE_DRAW_RTL) != 0;
    int32_t lightIx;
    const float3 L =
        sample_light<REF>(s, rng, rtl, I, sf.N, lightProb, lightPdf, lightRadiance, lightDist, lightIx);

    const float3 wow = -D;
    const float3 wo = normalize(make_float3(dot(wow, sf.T), dot(wow, sf.B), dot(wow, sf.N)));
    const float3 wi = normalize(make_float3(dot(L, sf.T), dot(L, sf.B), dot(L, sf.N)));
    if (vi) {
        vi->wo = wo;
        vi->wiLight = wi;
        vi->lightIx = lightIx;
    }

    float r0, r1;
    draw2(rng, rtl, r0, r1);
    ClosureResult c;
    if (closure == TR_CLOSURE_DISNEY)
        c = disney_closure<REF>(wo, wi, T, m, r0, r1, lightPdf > kEpsilon);
    else if (closure == TR_CLOSURE_DIFFUSE)
        c = diffuse_closure(wo, wi, T, m, r0, r1);
    else
        c = lambert_closure(wo, wi, T, m, r0, r1);

    if ((lightPdf > kEpsilon) && (c.shPdf > kEpsilon) && ((c.extFlags & kFlagSpecular) == 0)) {
        const float3 shadowT = (c.shT * lightRadiance) * fdiv(1.f, lightProb * lightPdf + c.shPdf);
        wantShadow = true;
        sh[0] = f4(I, __uint_as_float(pathIx));
        sh[1] = f4(L, lightDist);
        // a batch shadow ray carries its item's BVH root in T.w
        sh[2] = f4(safe_color(shadowT, st.maxColor),
                   BATCH ? u2f(item_root(f, batch_item_of(__float_as_uint(D4.w)))) : 0.f);
    }

    if (vi)
        vi->wiExt = c.extWi;
    if (c.extPdf > kEpsilon && (!BATCH || bounce + 1u < st.maxDepth)) {
        float3 tp = c.extT * fdiv(1.f, fabsf(c.extPdf));
        if (bounce >= st.rrStart) {
            const float rr = fminf(1.0f, fmaxf(tp.x, fmaxf(tp.y, tp.z)));
            if (rr < rng.next())
                return false;
            tp *= fdiv(1.f, rr);
        }
        const float3 nd = normalize((c.extWi.x * sf.T) + (c.extWi.y * sf.B) + (c.extWi.z * sf.N));
        if (c.extFlags & kFlagSpecular)
            flags |= kFlagSpecular;
        else
            flags &= ~kFlagSpecular;
        wantExt = true;
        ext[0] = f4(I, __uint_as_float(BATCH ? pathIx : pack_path(pathIx, flags)));
        ext[1] = f4(nd, __uint_as_float(BATCH ? batch_pack(bounce + 1u, flags, batch_item_of(__float_as_uint(D4.w)))
                                              : pack_normal(sf.N)));
        ext[2] = f4(fixnan(tp), c.extPdf);
    }
    return false;
}

// Dynamic shared memory of the shade kernel per thread: two staging buffers of
// the path state's three planes and the hit record.
constexpr uint32_t kShadeStageBytes = 2u * 4u * sizeof(float4);

// Blocks of 64 or 128 threads (LaunchShape::shadeThreads; dynamic shared memory
// of kShadeStageBytes per thread for the input staging), at most 96 registers.
template <bool REF, bool BATCH, bool TEX = false>
__global__ void __launch_bounds__(128, 5) shade_kernel(SceneView s, FrameView f, Settings st, uint32_t bounce)
{
    const uint32_t count = BATCH ? __ldcg(&f.batch->hits) : __ldcg(f.counters + kHitCounterBase + bounce);
    const float4* __restrict__ in = f.state[1];
    float4* __restrict__ out = f.state[0];
    const uint32_t cap = f.capacity;
    const uint32_t sc = *f.sampleCount;
    const uint32_t wh = f.resX * f.resY;
    uint32_t* extCounter = BATCH ? &f.batch->survivors : f.counters + bounce + 1u;
    uint32_t* shCounter = BATCH ? &f.batch->shadows : f.counters + kShadowCounterBase + bounce;
    const uint32_t lane = lane_id();
    const uint32_t warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t warpStride = (gridDim.x * blockDim.x) >> 5;
    // The next item's path state and hit record are copied (cp.async) while
    // this item is shaded. Two buffers: the one refilled was read an iteration
    // earlier, by loads whose values that iteration's shading consumed, so the
    // copy cannot overtake them.
    // stage[(b * 4 + plane) * blockDim.x + thread]: two buffers of the state's
    // three planes and the hit record
    extern __shared__ float4 stage[];
    const uint32_t tid = threadIdx.x;
    const uint32_t bd = blockDim.x;
    uint32_t buf = 0;
    auto at = [&](uint32_t b, uint32_t plane) -> float4* { return stage + (b * 4u + plane) * bd + tid; };
    auto fetch = [&](uint32_t k, uint32_t b) {
        const uint32_t i = f.hitOrder ? __ldcs(f.hitOrder + k) : k;
        cp_async16(at(b, 0), in + i);
        cp_async16(at(b, 1), in + i + cap);
        cp_async16(at(b, 2), in + i + 2 * cap);
        cp_async16(at(b, 3), f.hits + i);
        cp_async_commit();
    };
    if (warpGlobal * 32u + lane < count)
        fetch(warpGlobal * 32u + lane, 0u);

    for (uint32_t base = warpGlobal * 32u; base < count; base += warpStride * 32u) {
        const uint32_t k = base + lane;
        bool wantExt = false, wantShadow = false, emitted = false;
        float4 ext[3], sh[3];
        if (k < count) {
            cp_async_wait_all();
            const float4 O4 = *at(buf, 0);
            const float4 D4 = *at(buf, 1);
            const float4 T4 = *at(buf, 2);
            const float4 h = *at(buf, 3);
            const uint4 hd = make_uint4(__float_as_uint(h.x), __float_as_uint(h.y), __float_as_uint(h.z),
                                        __float_as_uint(h.w));
            buf ^= 1u;
            if (k + warpStride * 32u < count)
                fetch(k + warpStride * 32u, buf);
            const uint32_t pathIx = path_ix(__float_as_uint(O4.w));
            if (BATCH) {
                // O.w is the sample id, D.w the path's bounce and flags
                const uint32_t id = __float_as_uint(O4.w);
                const uint32_t pathBounce = batch_bounce(__float_as_uint(D4.w));
                const BatchSample bs = batch_sample_in(f, id, batch_item_of(__float_as_uint(D4.w)));
                const SceneView si = item_scene(s, f.items[bs.item]);
                CounterRng rng;
                rng.init(bs.pixel, sc + bs.sample, pathBounce + 1u, st.seed);
                emitted = shade_path<false, CounterRng, TEX, true>(si, f, st, pathBounce, sc, O4, D4, T4, hd, rng,
                                                                   wantExt, ext, wantShadow, sh);
            } else if (REF) {
                RefRng rng{tea2(st.seed + pathIx, sc + bounce + 1u)};
                emitted = shade_path<REF, RefRng, TEX>(s, f, st, bounce, sc, O4, D4, T4, hd, rng, wantExt, ext,
                                                       wantShadow, sh);
            } else {
                CounterRng rng;
                rng.init(pathIx % wh, sc + pathIx / wh, bounce + 1u, st.seed);
                emitted = shade_path<REF, CounterRng, TEX>(s, f, st, bounce, sc, O4, D4, T4, hd, rng, wantExt, ext,
                                                           wantShadow, sh);
            }
        }
        if (st.flags & TR_FLAG_COUNT_TRAVERSAL)
            add_count(f.traversal + 4, emitted ? 1u : 0u);
        uint32_t shSlot, exSlot;
        warp_append2(shCounter, wantShadow, shSlot, extCounter, wantExt, exSlot);
        if (wantShadow) {
            __stcs(f.shadow + shSlot, sh[0]);
            __stcs(f.shadow + shSlot + cap, sh[1]);
            __stcs(f.shadow + shSlot + 2 * cap, sh[2]);
        }
        if (wantExt) {
            __stcs(out + exSlot, ext[0]);
            __stcs(out + exSlot + cap, ext[1]);
            __stcs(out + exSlot + 2 * cap, ext[2]);
        }
    }
}

// Material sort of the hit queue (optional, chosen by the tuner): a counting
// sort by material index so that the lanes of a shade warp mostly share one
// material record and one closure branch. Histogram in shared memory per
// block, one exclusive scan, then a scatter with one atomic per (warp,
// material). The order inside a material is arbitrary; each path's result
// does not depend on it.
constexpr uint32_t kSortSmemBins = 8192;

__global__ void __launch_bounds__(256) sort_histogram_kernel(SceneView s, FrameView f, SortView sv, uint32_t bounce)
{
    __shared__ uint32_t hist[kSortSmemBins];
    const bool local = sv.bins <= kSortSmemBins;
    if (local) {
        for (uint32_t b = threadIdx.x; b < sv.bins; b += blockDim.x)
            hist[b] = 0u;
        __syncthreads();
    }
    const uint32_t count = __ldcg(f.counters + kHitCounterBase + bounce);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t key = __ldg(s.matIdx + f.hits[i].z);
        sv.keys[i] = key;
        if (local)
            atomicAdd(&hist[key], 1u);
        else
            atomicAdd(sv.counts + key, 1u);
    }
    if (local) {
        __syncthreads();
        for (uint32_t b = threadIdx.x; b < sv.bins; b += blockDim.x)
            if (hist[b])
                atomicAdd(sv.counts + b, hist[b]);
    }
}

// Exclusive scan of the counts into the cursors (one block), counts zeroed for
// the next bounce.
__global__ void __launch_bounds__(1024) sort_scan_kernel(SortView sv)
{
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0)
        carry = 0u;
    __syncthreads();
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    for (uint32_t base = 0; base < sv.bins; base += blockDim.x) {
        const uint32_t b = base + threadIdx.x;
        const uint32_t v = b < sv.bins ? sv.counts[b] : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, x, o);
            if (lane >= uint32_t(o))
                x += y;
        }
        if (lane == 31)
            warpSums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warpSums[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(kFull, w, o);
                if (lane >= uint32_t(o))
                    w += y;
            }
            warpSums[lane] = w;
        }
        __syncthreads();
        const uint32_t prefix = carry + (warp ? warpSums[warp - 1] : 0u) + x - v;
        if (b < sv.bins) {
            sv.cursor[b] = prefix;
            sv.counts[b] = 0u;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1)
            carry = prefix + v;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) sort_scatter_kernel(FrameView f, SortView sv, uint32_t bounce)
{
    const uint32_t count = __ldcg(f.counters + kHitCounterBase + bounce);
    const uint32_t lane = lane_id();
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < count;
         base += gridDim.x * blockDim.x) {
        const uint32_t i = base + lane;
        const uint32_t key = i < count ? sv.keys[i] : 0xffffffffu;
        const uint32_t peers = __match_any_sync(kFull, key);
        const uint32_t leader = __ffs(peers) - 1u;
        uint32_t pos = 0;
        if (lane == leader && key != 0xffffffffu)
            pos = atomicAdd(sv.cursor + key, __popc(peers));
        pos = __shfl_sync(kFull, pos, leader);
        if (key != 0xffffffffu)
            sv.order[pos + __popc(peers & ((1u << lane) - 1u))] = i;
    }
}

// Any hit of the bounce's shadow queue over [eps, dist - 2 eps]; an unoccluded
// ray adds its radiance to its path. Same lane refill as extend_kernel.
// Blocks of 64 or 128 threads (LaunchShape::traversalThreads): the kernel works per warp.
// One-level scenes: 56 registers, 9 blocks of 128 threads per SM (the kernel is bound by
// the latency of its node fetches; 31.3 against 33.1 ms of shadow rays per 1080p, 64 spp
// heightfield step at 72 registers and 7 blocks). Two-level traversal holds more state and
// keeps its own register count (it would spill 100-210 bytes at 56).
template <bool COUNT, bool BATCH, bool TL, int LAYOUT = kLayoutScene>
__global__ void __launch_bounds__(128, TL ? 1 : 9) connect_kernel(SceneView s, FrameView f, Settings st,
                                                                   uint32_t bounce)
{
    const uint32_t count = BATCH ? __ldcg(&f.batch->connectQueue) : __ldcg(f.counters + kShadowCounterBase + bounce);
    const uint32_t cap = f.capacity;
    uint32_t* work = BATCH ? &f.batch->connectWork : f.counters + kConnectWorkBase + bounce;
    const uint32_t lane = lane_id();
    TraversalCounts cnt{0, 0};
    uint32_t visibleCnt = 0;
    typename TravOf<TL>::type t;
    uint2 stack[kTraversalStack];
    uint32_t ray = 0, pathIx = 0;
    bool alive = false, more = true;
    while (true) {
        const uint32_t idle = __ballot_sync(kFull, !alive && more);
        if (idle) {
            const uint32_t leader = __ffs(idle) - 1u;
            uint32_t base = 0;
            if (lane == leader)
                base = atomicAdd(work, __popc(idle));
            base = __shfl_sync(kFull, base, leader);
            if (!alive && more) {
                const uint32_t i = base + __popc(idle & ((1u << lane) - 1u));
                if (i < count) {
                    const float4 O4 = __ldcs(f.shadow + i);
                    const float4 L4 = __ldcs(f.shadow + i + cap);
                    ray = i;
                    pathIx = __float_as_uint(O4.w);
                    const uint32_t root =
                        BATCH ? __float_as_uint(__ldcs(reinterpret_cast<const float*>(f.shadow + i + 2 * cap) + 3))
                              : 0u;
                    traversal_begin(t, f3(O4), f3(L4), st.rayEpsilon, L4.w - (2 * st.rayEpsilon), root);
                    alive = true;
                } else {
                    more = false;
                }
            }
        }
        if (!__any_sync(kFull, alive))
            break;
        uint32_t active;
        do {
            if (alive && traversal_step<true, COUNT, LAYOUT>(t, stack, s, &cnt)) {
                if (!base(t).ok)
                    atomicOr(f.errorFlag, 1u);
                if (base(t).hitSlot == 0xffffffffu) {
                    const float4 T4 = __ldcs(f.shadow + ray + 2 * cap);
                    float4 r = f.radiance[pathIx];
                    f.radiance[pathIx] = make_float4(r.x + T4.x, r.y + T4.y, r.z + T4.z, r.w);
                    if (COUNT)
                        ++visibleCnt;
                }
                alive = false;
            }
            active = __ballot_sync(kFull, alive);
        } while (uint32_t(__popc(active)) >= st.refillBelow);
    }
    if (COUNT) {
        add_counts(f.traversal + 2, cnt);
        add_count(f.traversal + 5, visibleCnt);
    }
}

// Sums each pixel's samples in sample order into the accumulator and writes
// colors = accumulator / sampleCount (FinalizeFrame; the film initialisation
// of optix.cu:181-188 happens here: a frame with sampleCount == 0 overwrites).
__global__ void __launch_bounds__(256) finalize_kernel(FrameView f, Settings st)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t wh = f.resX * f.resY;
    if (p >= wh)
        return;
    const uint32_t sc = *f.sampleCount;
    float3 sum = f3(0.f);
    for (uint32_t k = 0; k < st.multiSample; ++k) {
        const float4 r = f.radiance[p + k * wh];
        sum = sum + f3(r);
    }
    float4 acc = sc == 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : f.accumulator[p];
    acc = make_float4(acc.x + sum.x, acc.y + sum.y, acc.z + sum.z, acc.w + float(st.multiSample));
    f.accumulator[p] = acc;
    const float n = float(sc + st.multiSample);
    f.colors[p] = make_float4(acc.x / n, acc.y / n, acc.z / n, acc.w / n);
}

// ------------------------------------------------------------------ debug render modes
// The reference's other shade kernels (Tracer/CUDA/GPU/Shade/*.h except
// PathTracing.h), run over the whole bounce queue with hits stored by queue
// slot (no compaction: the ambient-occlusion and wireframe modes act on
// missed rays too). Each path sets its radiance (one contribution per path).

// Closest hit of every ray of the bounce's queue (state[bounce & 1]); the
// wireframe mode re-aims secondary rays at a jittered point of the pixel as
// the Secondary raygen program does (optix.cu:292-300).
__global__ void __launch_bounds__(128) debug_extend_kernel(SceneView s, FrameView f, Camera cam, Settings st,
                                                           uint32_t bounce)
{
    const uint32_t count = queue_length(f, bounce);
    float4* q = f.state[bounce & 1u];
    const uint32_t cap = f.capacity;
    const uint32_t sc = *f.sampleCount;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float4 O4 = q[i];
        float3 O = f3(O4), D = f3(q[i + cap]);
        const uint32_t pathIx = path_ix(__float_as_uint(O4.w));
        if (st.renderMode == kModeWireframe && bounce > 0) {
            const uint32_t wh = f.resX * f.resY;
            const uint32_t pixelIx = pathIx % wh;
            RefRng rng{tea2(st.seed + pathIx, (sc << 1) | 1u)};
            float T;
            camera_ray(cam, f.resX, f.resY, pixelIx % f.resX, pixelIx / f.resX, rng,
                       (st.flags & TR_FLAG_REFERENCE_DRAW_RTL) != 0, O, D, T);
        }
        float tmax = kDstMax;
        uint32_t slot = 0xffffffffu, inst = 0;
        float u = 0.f, v = 0.f;
        if (!traverse<false>(s, O, D, st.rayEpsilon, tmax, slot, u, v, nullptr, &inst))
            atomicOr(f.errorFlag, 1u);
        f.hits[i] = slot != 0xffffffffu
                        ? make_uint4(encode_bary(u, v), inst, __float_as_uint(__ldg(s.bvhTris + 3u * slot).w),
                                     __float_as_uint(tmax))
                        : make_uint4(0u, 0xffffffffu, 0xffffffffu, __float_as_uint(kDstMax));
    }
}

// RayPick raygen (optix.cu:345-377): the camera ray of pixel (x, resY - y) with the
// random stream seeded 0, traced closest-hit; result = RayPickResult (7 words:
// camera position, instIx, direction, primIx, tmax).
__global__ void __launch_bounds__(32) pick_ray_kernel(SceneView s, Camera cam, Settings st, uint32_t resX,
                                                      uint32_t resY, int x, int y, float* result, uint32_t* errorFlag)
{
    if (threadIdx.x != 0)
        return;
    RefRng rng{0u};
    float3 O, D;
    float T;
    camera_ray(cam, resX, resY, x, int(resY) - y, rng, (st.flags & TR_FLAG_REFERENCE_DRAW_RTL) != 0, O, D, T);
    uint32_t inst = 0xffffffffu, prim = 0xffffffffu;
    float tmax = kDstMax;
    if (T > 0.f) {
        uint32_t slot = 0xffffffffu, hitInst = 0;
        float u = 0.f, v = 0.f;
        if (!traverse<false>(s, O, D, st.rayEpsilon, tmax, slot, u, v, nullptr, &hitInst))
            atomicOr(errorFlag, 1u);
        if (slot != 0xffffffffu) {
            inst = hitInst;
            prim = __float_as_uint(__ldg(s.bvhTris + 3u * slot).w);
        }
    }
    result[0] = cam.pos.x;
    result[1] = cam.pos.y;
    result[2] = cam.pos.z;
    result[3] = __uint_as_float(inst);
    result[4] = D.x;
    result[5] = D.y;
    result[6] = D.z;
    result[7] = __uint_as_float(prim);
    result[8] = tmax;
}

// OrthonormalBase + SampleCosineHemisphere (CudaUtility.h:182-199, 271-292)
__device__ __forceinline__ float3 cosine_hemisphere(const float3& n, float r0, float r1)
{
    float3 b = fabsf(n.x) > fabsf(n.y) ? make_float3(-n.y, n.x, 0.f) : make_float3(0.f, -n.z, n.y);
    b = normalize(b);
    const float3 t = cross(b, n);
    float sinPhi, cosPhi;
    sincosf(2.0f * kPi * r0, &sinPhi, &cosPhi);
    const float rb = sqrtf(1.f - r1);
    const float3 l = make_float3(cosPhi * rb, sinPhi * rb, sqrtf(r1));
    return l.x * t + l.y * b + l.z * n;
}

// IdToColor (CudaUtility.h:14-27): bits of id spread over the three channels
__device__ __forceinline__ float3 id_to_color(uint32_t id)
{
    uint32_t c[3];
    for (uint32_t i = 0; i < 3; ++i) {
        c[i] = (id >> i) & 0x249249u;
        c[i] = ((c[i] << 1) | (c[i] >> 3)) & 0x0C30C3u;
        c[i] = ((c[i] << 2) | (c[i] >> 6)) & 0x00F00Fu;
        c[i] = ((c[i] << 4) | (c[i] >> 12)) & 0x0000FFu;
    }
    return make_float3(c[0] * (1.f / 255.f), c[1] * (1.f / 255.f), c[2] * (1.f / 255.f));
}

__global__ void __launch_bounds__(128) debug_shade_kernel(SceneView s, FrameView f, Camera cam, Settings st,
                                                          uint32_t bounce)
{
    const uint32_t count = queue_length(f, bounce);
    const float4* in = f.state[bounce & 1u];
    float4* out = f.state[(bounce + 1u) & 1u];
    const uint32_t cap = f.capacity;
    const uint32_t sc = *f.sampleCount;
    const uint32_t wh = f.resX * f.resY;
    const bool rtl = (st.flags & TR_FLAG_REFERENCE_DRAW_RTL) != 0;
    const bool aov = (st.flags & TR_FLAG_WRITE_AOVS) != 0;
    uint32_t* extCounter = f.counters + bounce + 1u;
    const uint32_t mode = st.renderMode;
    const bool ao = mode == kModeAO || mode == kModeAOShading;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < count;
         base += gridDim.x * blockDim.x) {
        const uint32_t i = base + lane_id();
        bool wantExt = false;
        float4 ext[3];
        if (i < count) {
            const float4 O4 = in[i];
            const float4 D4 = in[i + cap];
            const uint4 hd = f.hits[i];
            const uint32_t pathIx = path_ix(__float_as_uint(O4.w));
            const uint32_t pixelIx = pathIx % wh;
            const bool hit = hd.z != 0xffffffffu;
            const float tmax = __uint_as_float(hd.w);
            float3 c = f3(0.f);
            bool set = false;
            if (ao && bounce > 0) {
                // the occlusion ray: 1 beyond aoDist (or on a miss), else tmax / aoDist
                const float z = tmax > st.aoDist ? 1.f : tmax / st.aoDist;
                c = mode == kModeAO ? make_float3(z, z, z) : f3(in[i + 2 * cap]) * z;
                set = true;
            } else if (mode == kModeWireframe) {
                if (bounce == 0) {
                    // trace a second, jittered ray; keep this hit's primitive
                    wantExt = true;
                    ext[0] = f4(f3(O4), __uint_as_float(pack_path(pathIx, 0)));
                    ext[1] = f4(f3(D4), 0.f);
                    ext[2] = make_float4(0.f, 0.f, 0.f, __uint_as_float(hd.z));
                } else if (__float_as_uint(in[i + 2 * cap].w) == hd.z) {
                    c = make_float3(1.f, 1.f, 1.f);
                    set = true;
                }
            } else if (mode == kModeZDepth) {
                if (hit) {
                    const float z = fminf(fmaxf(tmax * dot(f3(D4), cam.forward) / st.zDepthMax, 0.f), 1.f);
                    c = make_float3(z, z, z);
                    set = true;
                }
            } else if (mode == kModeObjectID) {
                if (hit) {
                    c = id_to_color(hd.y + 1u);
                    set = true;
                }
            } else if (hit && bounce == 0) {
                const float2 bary = decode_bary(hd.x);
                const bool fix = ao;
                const Surface sf = surface_at<true>(s, hd.y, hd.z, bary, fix ? f3(D4) : f3(0.f));
                uint32_t closure, emissiveFlag, texMask;
                HitMat m = load_material(s.materials, sf.matIx, closure, emissiveFlag, &texMask);
                if (texMask)
                    apply_textures(s, sf.matIx, texMask, sf.uv, m, emissiveFlag);
                if (ao) {
                    uint32_t seed = tea2(st.seed + pathIx, mode == kModeAO ? bounce + 1u : sc + bounce + 1u);
                    if (mode == kModeAO)
                        seed ^= sc;  // rot_seed (random.h:69-72)
                    RefRng rng{seed};
                    float r0, r1;
                    draw2(rng, rtl, r0, r1);
                    const float3 I = f3(O4) + f3(D4) * tmax;
                    wantExt = true;
                    ext[0] = f4(I, __uint_as_float(pack_path(pathIx, 0)));
                    ext[1] = f4(cosine_hemisphere(sf.N, r0, r1), 0.f);
                    const float3 T = mode == kModeAO ? make_float3(1.f, 1.f, 1.f) : m.diffuse;
                    ext[2] = f4(T, 0.f);
                    c = T;  // the value of an occlusion ray that escapes
                    set = true;
                    if (aov && pathIx < wh) {
                        f.albedo[pixelIx] = f4(mode == kModeAO ? make_float3(1.f, 1.f, 1.f) : m.diffuse, 0.f);
                        f.normals[pixelIx] = f4(sf.N, 0.f);
                    }
                } else {
                    set = true;
                    switch (mode) {
                    case kModeBitangent: c = (sf.B + make_float3(1.f, 1.f, 1.f)) * 0.5f; break;
                    case kModeGeometricNormal: c = (sf.Ng + make_float3(1.f, 1.f, 1.f)) * 0.5f; break;
                    case kModeShadingNormal: c = (sf.N + make_float3(1.f, 1.f, 1.f)) * 0.5f; break;
                    case kModeTangent: c = (sf.T + make_float3(1.f, 1.f, 1.f)) * 0.5f; break;
                    case kModeMaterialID: c = id_to_color(sf.matIx + 1u); break;
                    case kModeTextureCoordinate: {
                        const uint32_t ti = (s.instInfo ? __ldg(&s.instInfo[hd.y].y) : 0u) + hd.z;
                        const TriShade& tri = s.tris[ti];
                        const float2 u0 = make_float2(h2f(tri.uv0x), h2f(tri.uv0y));
                        const float2 u1 = make_float2(h2f(tri.uv1x), h2f(tri.uv1y));
                        const float2 u2 = make_float2(h2f(tri.uv2x), h2f(tri.uv2y));
                        const float2 uv = make_float2(u0.x + ((u1.x - u0.x) * bary.x) + ((u2.x - u0.x) * bary.y),
                                                      u0.y + ((u1.y - u0.y) * bary.x) + ((u2.y - u0.y) * bary.y));
                        c = make_float3(uv.x, uv.y, 0.f);
                        break;
                    }
                    case kModeMaterialProperty:
                        switch (st.renderFlags) {  // MaterialPropertyIds
                        case 0: c = make_float3(m.anisotropic, m.anisotropic, m.anisotropic); break;
                        case 1: c = make_float3(m.clearcoat, m.clearcoat, m.clearcoat); break;
                        case 2: c = make_float3(m.clearcoatGloss, m.clearcoatGloss, m.clearcoatGloss); break;
                        case 3: c = m.diffuse; break;
                        case 4: c = m.emissive; break;
                        case 5: c = make_float3(m.metallic, m.metallic, m.metallic); break;
                        case 6:  // GetColor(Normal): the map's RGB, else GetColor's default
                            c = (texMask & (1u << TR_PROP_NORMAL))
                                    ? tex_rgb(__ldg(&s.texSlots[sf.matIx].tex[TR_PROP_NORMAL]), sf.uv)
                                    : make_float3(1.f, 1.f, 1.f);
                            break;
                        case 7: c = make_float3(m.roughness, m.roughness, m.roughness); break;
                        case 8: c = make_float3(m.sheen, m.sheen, m.sheen); break;
                        case 9: c = make_float3(m.sheenTint, m.sheenTint, m.sheenTint); break;
                        case 10: c = make_float3(m.specular, m.specular, m.specular); break;
                        case 11: c = make_float3(m.specularTint, m.specularTint, m.specularTint); break;
                        case 12: c = make_float3(m.subsurface, m.subsurface, m.subsurface); break;
                        default: c = make_float3(1.f, 0.f, 1.f); break;
                        }
                        break;
                    default: set = false; break;
                    }
                }
            }
            if (set)
                f.radiance[pathIx] = f4(safe_color(c, st.maxColor), 0.f);
        }
        const uint32_t slot = warp_append(extCounter, wantExt);
        if (wantExt) {
            out[slot] = ext[0];
            out[slot + cap] = ext[1];
            out[slot + 2 * cap] = ext[2];
        }
    }
}

// Batched rendering: one iteration's plan. Sums the iteration that ended into
// the totals, hands its shadow rays to this iteration's connect, carries its
// surviving paths over (the first `carried` entries of the extend queue) and
// fills the rest of the pool with new samples from the cursor; with a conditional handle (graph replay) the batch's while loop goes
// on as long as the new iteration has rays to trace. Every path ends within
// max_depth iterations, so a round needs at most samples * max_depth
// iterations; `limit` (above that) ends the loop with the error word set
// should the counts ever say otherwise.
__global__ void batch_plan_kernel(BatchState* __restrict__ bs, uint32_t pool, uint32_t end, uint32_t limit,
                                  uint32_t* __restrict__ errorFlag, cudaGraphConditionalHandle loop, int32_t useLoop)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    BatchState s = *bs;
    s.end = end;
    s.extendRays += s.queue;
    s.shadowRays += s.shadows;
    s.hitRays += s.hits;
    s.connectQueue = s.shadows;
    const uint32_t carried = s.survivors;  // <= the last queue length <= pool
    const uint32_t room = pool - carried;
    const uint32_t left = s.end - s.cursor;
    const uint32_t fresh = left < room ? left : room;
    s.carried = carried;
    s.freshBase = s.cursor;
    s.cursor += fresh;
    s.queue = carried + fresh;
    if (s.queue && s.iterations >= limit) {
        s.queue = 0;
        atomicOr(errorFlag, 2u);
    }
    s.survivors = 0;
    s.hits = 0;
    s.shadows = 0;
    s.extendWork = 0;
    s.connectWork = 0;
    if (s.queue)
        s.iterations++;
    *bs = s;
    if (useLoop)
        cudaGraphSetConditional(loop, s.queue ? 1u : 0u);
}

// Batched rendering: every pixel of the round's items, its samples summed in
// sample order (as finalize_kernel sums one frame's multi_sample samples), added
// to the accumulator (which the first samples overwrite: *f.sampleCount == 0)
// and colors = accumulator / (samples before + spp).
__global__ void __launch_bounds__(256) batch_finalize_kernel(FrameView f, uint32_t pixelBegin, uint32_t pixelEnd)
{
    const uint32_t p = pixelBegin + blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pixelEnd)
        return;
    uint32_t lo = 0, hi = f.itemCount;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&f.items[mid].pixelBase) <= p)
            lo = mid;
        else
            hi = mid;
    }
    const BatchItem& it = f.items[lo];
    const uint32_t spp = it.spp;
    const float4* r = f.radiance + it.sampleBase + size_t(p - it.pixelBase) * spp;
    // in sample order; a thread's samples are consecutive, the lanes of a warp
    // spp float4 apart, so two loads in flight per step and the lines kept in L1
    // for the thread's next samples
    float3 sum = f3(0.f);
    uint32_t k = 0;
    for (; k + 1u < spp; k += 2u) {
        const float4 a = __ldg(r + k);
        const float4 b = __ldg(r + k + 1u);
        sum = sum + f3(a);
        sum = sum + f3(b);
    }
    if (k < spp)
        sum = sum + f3(__ldg(r + k));
    const uint32_t sc = *f.sampleCount;
    float4 acc = sc == 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : f.accumulator[p];
    acc = make_float4(acc.x + sum.x, acc.y + sum.y, acc.z + sum.z, acc.w + float(spp));
    f.accumulator[p] = acc;
    const float n = float(sc + spp);
    f.colors[p] = make_float4(acc.x / n, acc.y / n, acc.z / n, acc.w / n);
}

// Adds each lane's gradient slots [first, last) to the row of its key
// (material); key == ~0: nothing to add. Lanes that share a key are summed by
// a butterfly over the warp, one distinct key at a time, and the first lane of
// the key adds the sums: with SMEM to the warp's private copy in shared memory
// (plain read-modify-write: only that lane writes there), else with global
// atomics.
template <bool SMEM>
__device__ __forceinline__ void warp_add_grads(float* __restrict__ dst, uint32_t key, const float (&g)[kGradSlots],
                                               int first, int last)
{
    const uint32_t lane = lane_id();
    uint32_t pending = __ballot_sync(kFull, key != 0xffffffffu);
    while (pending) {
        const uint32_t leader = __ffs(pending) - 1u;
        const uint32_t cur = __shfl_sync(kFull, key, leader);
        const bool mine = key == cur;
        pending &= ~__ballot_sync(kFull, mine);
#pragma unroll
        for (int k = 0; k < kGradSlots; ++k) {
            if (k < first || k >= last)
                continue;
            float v = mine ? g[k] : 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                v += __shfl_xor_sync(kFull, v, o);
            if (lane == leader && v != 0.f) {
                float* a = dst + size_t(cur) * kGradSlots + k;
                if (SMEM)
                    *a += v;
                else
                    atomicAdd(a, v);
            }
        }
    }
}

// Shared memory of one adjoint block: one copy of the gradient table per warp.
constexpr uint32_t kAdjointThreads = 128;
constexpr uint32_t kAdjointWarps = kAdjointThreads / 32;
// Largest dynamic shared memory without the opt-in attribute: 4 copies of
// 9 floats per material, up to 341 materials; more use global atomics.
constexpr size_t kAdjointSmemMax = 48 * 1024;

// Gradient table of an adjoint block: the warp's private copy in shared
// memory (zeroed here) when SMEM, else the global table.
template <bool SMEM>
__device__ __forceinline__ float* grad_table_begin(float* sgrad, const AdjointView& a)
{
    if (!SMEM)
        return a.grads;
    const uint32_t rows = a.materialCount * kGradSlots;
    for (uint32_t i = threadIdx.x; i < kAdjointWarps * rows; i += blockDim.x)
        sgrad[i] = 0.f;
    __syncthreads();
    return sgrad + (threadIdx.x >> 5) * rows;
}

// Adds the block's shared-memory copies to the global table, one atomic per
// non-zero entry.
template <bool SMEM>
__device__ __forceinline__ void grad_table_end(const float* sgrad, const AdjointView& a)
{
    if (!SMEM)
        return;
    __syncthreads();
    const uint32_t rows = a.materialCount * kGradSlots;
    for (uint32_t i = threadIdx.x; i < rows; i += blockDim.x) {
        float v = 0.f;
#pragma unroll
        for (uint32_t w = 0; w < kAdjointWarps; ++w)
            v += sgrad[w * rows + i];
        if (v != 0.f)
            atomicAdd(a.grads + i, v);
    }
}

__device__ __forceinline__ float3 path_delta(const FrameView& f, const AdjointView& a, uint32_t pathIx)
{
    const float4 pg = a.pixelGrad[pathIx % (f.resX * f.resY)];
    return make_float3(pg.x * a.scale, pg.y * a.scale, pg.z * a.scale);
}

// g[k] += sum_c w_c * (d f_c / d theta_k) / f_c
__device__ __forceinline__ void add_log_derivative(float (&g)[kGradSlots], const Vec3<Dual>& fv, const float3& w)
{
    const Dual* fc[3] = {&fv.x, &fv.y, &fv.z};
    const float wc[3] = {w.x, w.y, w.z};
#pragma unroll
    for (int c = 0; c < 3; ++c)
        if (wc[c] != 0.f && fc[c]->v != 0.f) {
            const float r = wc[c] / fc[c]->v;
#pragma unroll
            for (int k = 0; k < kGradParams; ++k)
                g[k] += r * fc[c]->d[k];
        }
}

// Path-replay adjoint (Vicini, Speierer, Jakob, "Path Replay Backpropagation",
// SIGGRAPH 2021) as a wavefront over the same queues as the forward frame:
// paths are regenerated from their random keys and re-traced by the forward
// extend kernel; the kernels below replace shade and connect. The gradient
// of the radiance that reached the camera through a closure value f is that
// radiance times d log f: for the light direction the vertex's NEE
// contribution, for the extend direction everything the path collected after
// the vertex. The latter is the path's total (the forward frame's per-path
// radiance) minus what was accounted for up to the vertex, so it is known
// when the path reaches its next vertex: the extend direction (wo, wi,
// material) is kept per path (pending) and its d log f is evaluated and
// weighted by ext_grad_kernel when the path's next hit is known.
__global__ void __launch_bounds__(256) adjoint_generate_kernel(FrameView f, Camera cam, Settings st, AdjointView a)
{
    const uint32_t pathIx = blockIdx.x * blockDim.x + threadIdx.x;
    if (pathIx >= f.pathCount)
        return;
    const uint32_t wh = f.resX * f.resY;
    const uint32_t pixelIx = pathIx % wh;
    const uint32_t sc = a.sampleBase;
    CounterRng rng;
    rng.init(pixelIx, sc + pathIx / wh, 0u, st.seed);
    float3 O, D;
    float T;
    camera_ray(cam, f.resX, f.resY, pixelIx % f.resX, pixelIx / f.resX, rng, false, O, D, T);
    const uint32_t cap = f.capacity;
    float4* s = f.state[0];
    s[pathIx] = f4(O, u2f(pack_path(pathIx, 0)));
    s[pathIx + cap] = f4(D, 0.f);
    s[pathIx + 2 * cap] = make_float4(T, T, T, 1.f);
    a.lrem[pathIx] = f.radiance[pathIx];
    a.pending[pathIx] = make_float4(0.f, 0.f, 0.f, __uint_as_float(0xffffffffu));
}

// Gradient of the previous vertex's extend direction, for the paths of the
// bounce's hit queue (launched after extend, before adjoint_shade_kernel
// takes this vertex's emission off the remaining radiance): the radiance
// still unaccounted for arrived through that direction.
template <bool SMEM>
__global__ void __launch_bounds__(kAdjointThreads) ext_grad_kernel(SceneView s, FrameView f, uint32_t bounce,
                                                                   AdjointView a)
{
    extern __shared__ float sgrad[];
    float* table = grad_table_begin<SMEM>(sgrad, a);
    const uint32_t count = __ldcg(f.counters + kHitCounterBase + bounce);
    const float4* __restrict__ in = f.state[1];
    const uint32_t cap = f.capacity;
    const uint32_t warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t warpStride = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warpGlobal * 32u; base < count; base += warpStride * 32u) {
        const uint32_t i = base + lane_id();
        float g[kGradSlots];
#pragma unroll
        for (int k = 0; k < kGradSlots; ++k)
            g[k] = 0.f;
        uint32_t key = 0xffffffffu;
        if (i < count) {
            const uint32_t pathIx = path_ix(__float_as_uint(__ldg(in + i).w));
            const float4 wo4 = a.pending[pathIx];
            const uint32_t matIx = __float_as_uint(wo4.w);
            if (matIx != 0xffffffffu) {
                const float3 delta = path_delta(f, a, pathIx);
                const float3 lrem = f3(a.lrem[pathIx]);
                const float3 w = make_float3(delta.x * lrem.x, delta.y * lrem.y, delta.z * lrem.z);
                if (w.x != 0.f || w.y != 0.f || w.z != 0.f) {
                    const float4 wi4 = a.pending[pathIx + cap];
                    uint32_t closure, emissiveFlag;
                    const HitMat m = load_material(s.materials, matIx, closure, emissiveFlag);
                    add_log_derivative(g, dual::closure_value(closure, m, f3(wo4), f3(wi4)), w);
                    key = matIx;
                }
            }
        }
        warp_add_grads<SMEM>(table, key, g, 0, kGradParams);
    }
    grad_table_end<SMEM>(sgrad, a);
}

// Shade of the replay over the hit queue: the emission gradients of an
// emissive hit; queues the NEE ray (with what the NEE gradient needs) and the
// extend ray (with its direction kept as the path's pending record) like the
// forward shade.
template <bool SMEM>
__global__ void __launch_bounds__(kAdjointThreads, 4) adjoint_shade_kernel(SceneView s, FrameView f, Settings st,
                                                                        uint32_t bounce, AdjointView a)
{
    extern __shared__ float sgrad[];
    float* table = grad_table_begin<SMEM>(sgrad, a);
    const uint32_t count = __ldcg(f.counters + kHitCounterBase + bounce);
    const float4* __restrict__ in = f.state[1];
    float4* __restrict__ out = f.state[0];
    const uint32_t cap = f.capacity;
    const uint32_t sc = a.sampleBase;
    const uint32_t wh = f.resX * f.resY;
    uint32_t* extCounter = f.counters + bounce + 1u;
    uint32_t* shCounter = f.counters + kShadowCounterBase + bounce;
    const uint32_t warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t warpStride = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warpGlobal * 32u; base < count; base += warpStride * 32u) {
        const uint32_t i = base + lane_id();
        bool wantExt = false, wantShadow = false;
        float4 ext[3], sh[3];
        float g[kGradSlots], ge[kGradSlots];
#pragma unroll
        for (int k = 0; k < kGradSlots; ++k)
            g[k] = ge[k] = 0.f;
        uint32_t key = 0xffffffffu, keyE = 0xffffffffu;
        uint32_t pathIx = 0;
        VertexInfo vi;
        vi.hit = false;
        if (i < count) {
            const float4 O4 = __ldcs(in + i);
            const float4 D4 = __ldcs(in + i + cap);
            const float4 T4 = __ldcs(in + i + 2 * cap);
            const uint4 hd = __ldcs(f.hits + i);
            pathIx = path_ix(__float_as_uint(O4.w));
            const float3 delta = path_delta(f, a, pathIx);
            float3 lrem = f3(a.lrem[pathIx]);
            const bool live = (delta.x != 0.f || delta.y != 0.f || delta.z != 0.f) &&
                              (lrem.x != 0.f || lrem.y != 0.f || lrem.z != 0.f);
            if (live) {
                CounterRng rng;
                rng.init(pathIx % wh, sc + pathIx / wh, bounce + 1u, st.seed);
                shade_path<false>(s, f, st, bounce, sc, O4, D4, T4, hd, rng, wantExt, ext, wantShadow, sh, &vi);
            }
            if (vi.hit && vi.emissive) {
                const float C[3] = {vi.emitted.x, vi.emitted.y, vi.emitted.z};
                const float E[3] = {vi.mat.emissive.x, vi.mat.emissive.y, vi.mat.emissive.z};
                const float dl[3] = {delta.x, delta.y, delta.z};
                const float Dc[3] = {vi.mat.diffuse.x, vi.mat.diffuse.y, vi.mat.diffuse.z};
                // emission = Emissive * diffuse (CudaMaterial.h:158): linear in both
                for (int c = 0; c < 3; ++c) {
                    if (E[c] > 0.f)
                        ge[kGEmR + c] = dl[c] * C[c] / E[c] * Dc[c];
                    if (Dc[c] > 0.f)
                        g[kGBaseR + c] = dl[c] * C[c] / Dc[c];
                }
                keyE = vi.matIx;
                key = vi.matIx;
                lrem = lrem - vi.emitted;
                a.lrem[pathIx] = f4(lrem, 0.f);
            } else if (vi.hit && wantExt) {
                // the extend direction, weighted when the path's next vertex is known
                a.pending[pathIx] = f4(vi.wo, __uint_as_float(vi.matIx));
                a.pending[pathIx + cap] = f4(vi.wiExt, 0.f);
            }
        }
        if (vi.emissive)
            wantExt = wantShadow = false;
        const uint32_t shSlot = warp_append(shCounter, wantShadow);
        if (wantShadow) {
            __stcs(f.shadow + shSlot, sh[0]);
            __stcs(f.shadow + shSlot + cap, sh[1]);
            __stcs(f.shadow + shSlot + 2 * cap, sh[2]);
            a.shadowAdj[shSlot] = f4(vi.wo, __uint_as_float(vi.matIx));
            a.shadowAdj[shSlot + cap] = f4(vi.wiLight, __int_as_float(vi.lightIx));
        }
        const uint32_t exSlot = warp_append(extCounter, wantExt);
        if (wantExt) {
            __stcs(out + exSlot, ext[0]);
            __stcs(out + exSlot + cap, ext[1]);
            __stcs(out + exSlot + 2 * cap, ext[2]);
        }
        warp_add_grads<SMEM>(table, key, g, 0, kGradParams);
        warp_add_grads<SMEM>(table, keyE, ge, kGEmR, kGradSlots);
    }
    grad_table_end<SMEM>(sgrad, a);
}

// Visibility of the replay's NEE rays (as connect_kernel): an unoccluded ray
// takes its contribution off the path's remaining radiance and is listed for
// nee_grad_kernel.
template <bool TL>
__global__ void __launch_bounds__(128) adjoint_connect_kernel(SceneView s, FrameView f, Settings st, uint32_t bounce,
                                                              AdjointView a)
{
    const uint32_t count = __ldcg(f.counters + kShadowCounterBase + bounce);
    const uint32_t cap = f.capacity;
    uint32_t* work = f.counters + kConnectWorkBase + bounce;
    uint32_t* visCounter = f.counters + kVisibleCounterBase + bounce;
    const uint32_t lane = lane_id();
    typename TravOf<TL>::type t;
    uint2 stack[kTraversalStack];
    uint32_t ray = 0, pathIx = 0;
    bool alive = false, more = true;
    while (true) {
        const uint32_t idle = __ballot_sync(kFull, !alive && more);
        if (idle) {
            const uint32_t leader = __ffs(idle) - 1u;
            uint32_t base = 0;
            if (lane == leader)
                base = atomicAdd(work, __popc(idle));
            base = __shfl_sync(kFull, base, leader);
            if (!alive && more) {
                const uint32_t i = base + __popc(idle & ((1u << lane) - 1u));
                if (i < count) {
                    const float4 O4 = __ldcs(f.shadow + i);
                    const float4 L4 = __ldcs(f.shadow + i + cap);
                    ray = i;
                    pathIx = __float_as_uint(O4.w);
                    traversal_begin(t, f3(O4), f3(L4), st.rayEpsilon, L4.w - (2 * st.rayEpsilon));
                    alive = true;
                } else {
                    more = false;
                }
            }
        }
        if (!__any_sync(kFull, alive))
            break;
        uint32_t active;
        do {
            bool visible = false;
            if (alive && traversal_step<true, false>(t, stack, s, nullptr)) {
                if (!base(t).ok)
                    atomicOr(f.errorFlag, 1u);
                if (base(t).hitSlot == 0xffffffffu) {
                    const float4 T4 = __ldcs(f.shadow + ray + 2 * cap);
                    const float4 r = a.lrem[pathIx];
                    a.lrem[pathIx] = make_float4(r.x - T4.x, r.y - T4.y, r.z - T4.z, r.w);
                    visible = true;
                }
                alive = false;
            }
            const uint32_t slot = warp_append(visCounter, visible);
            if (visible)
                a.visible[slot] = ray;
            active = __ballot_sync(kFull, alive);
        } while (uint32_t(__popc(active)) >= st.refillBelow);
    }
}

// Gradients of the visible NEE contributions: d log f of the light direction
// at the vertex, and the light's emission.
template <bool SMEM>
__global__ void __launch_bounds__(kAdjointThreads) nee_grad_kernel(SceneView s, FrameView f, uint32_t bounce,
                                                                   AdjointView a)
{
    extern __shared__ float sgrad[];
    float* table = grad_table_begin<SMEM>(sgrad, a);
    const uint32_t count = __ldcg(f.counters + kVisibleCounterBase + bounce);
    const uint32_t cap = f.capacity;
    const uint32_t warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t warpStride = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warpGlobal * 32u; base < count; base += warpStride * 32u) {
        const uint32_t i = base + lane_id();
        float g[kGradSlots], ge[kGradSlots];
#pragma unroll
        for (int k = 0; k < kGradSlots; ++k)
            g[k] = ge[k] = 0.f;
        uint32_t key = 0xffffffffu, keyE = 0xffffffffu;
        if (i < count) {
            const uint32_t ray = a.visible[i];
            const uint32_t pathIx = __float_as_uint(f.shadow[ray].w);
            const float3 C = f3(f.shadow[ray + 2 * cap]);
            const float4 wo4 = a.shadowAdj[ray];
            const float4 wi4 = a.shadowAdj[ray + cap];
            const uint32_t matIx = __float_as_uint(wo4.w);
            const int32_t lightIx = __float_as_int(wi4.w);
            const float3 delta = path_delta(f, a, pathIx);
            const float3 w = make_float3(delta.x * C.x, delta.y * C.y, delta.z * C.z);
            uint32_t closure, emissiveFlag;
            const HitMat m = load_material(s.materials, matIx, closure, emissiveFlag);
            add_log_derivative(g, dual::closure_value(closure, m, f3(wo4), f3(wi4)), w);
            key = matIx;
            if (lightIx >= 0) {
                const LightTri& Lt = s.lights[lightIx];
                const float E[3] = {Lt.radiance.x, Lt.radiance.y, Lt.radiance.z};
                const float wc[3] = {w.x, w.y, w.z};
                for (int c = 0; c < 3; ++c)
                    if (E[c] > 0.f)
                        ge[kGEmR + c] = wc[c] / E[c];
                keyE = __ldg(s.matIdx + Lt.triIx);
            }
        }
        warp_add_grads<SMEM>(table, key, g, 0, kGradParams);
        warp_add_grads<SMEM>(table, keyE, ge, kGEmR, kGradSlots);
    }
    grad_table_end<SMEM>(sgrad, a);
}

__global__ void advance_kernel(FrameView f, Settings st)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        *f.sampleCount += st.multiSample;
}

} // namespace

// ------------------------------------------------------------------ launchers
namespace {
// The scene as a traversal launch sees it: with the settings' bound on the
// node visits of one ray.
SceneView traced(const SceneView& s, const Settings& st)
{
    SceneView v = s;
    v.stepLimit = st.stepLimit ? st.stepLimit : kMaxTraversalSteps;
    return v;
}
} // namespace

cudaError_t launch_generate(const FrameView& f, const Camera& cam, const Settings& st, cudaStream_t stream)
{
    if (f.pathCount == 0)
        return cudaSuccess;
    const uint32_t blocks = (f.pathCount + 255u) / 256u;
    if (st.flags & TR_FLAG_REFERENCE_SAMPLING)
        generate_kernel<true, false><<<blocks, 256, 0, stream>>>(f, cam, st);
    else
        generate_kernel<false, false><<<blocks, 256, 0, stream>>>(f, cam, st);
    return cudaGetLastError();
}

template <bool PRIMARY>
void launch_extend_variant(const SceneView& s0, const FrameView& f, const Settings& st, uint32_t bounce,
                           const Camera& cam, const LaunchShape& shape, cudaStream_t stream)
{
    const SceneView s = traced(s0, st);
    const bool count = (st.flags & TR_FLAG_COUNT_TRAVERSAL) != 0;
    const uint32_t g = shape.extendBlocks;
    const uint32_t b = shape.traversalThreads;
    // one-level scenes: an instance per node layout
    auto oneLevel = [&](auto batchTag) {
        constexpr bool BATCH = decltype(batchTag)::value;
        if (s.quantNodes) {
            if (count)
                extend_kernel<true, BATCH, PRIMARY, false, kLayoutQuant><<<g, b, 0, stream>>>(s, f, st, bounce, cam);
            else
                extend_kernel<false, BATCH, PRIMARY, false, kLayoutQuant><<<g, b, 0, stream>>>(s, f, st, bounce, cam);
        } else {
            if (count)
                extend_kernel<true, BATCH, PRIMARY, false, kLayoutWide><<<g, b, 0, stream>>>(s, f, st, bounce, cam);
            else
                extend_kernel<false, BATCH, PRIMARY, false, kLayoutWide><<<g, b, 0, stream>>>(s, f, st, bounce, cam);
        }
    };
    auto twoLevel = [&](auto batchTag) {
        constexpr bool BATCH = decltype(batchTag)::value;
        if (!s.quantNodes) {
            if (count)
                extend_kernel<true, BATCH, PRIMARY, true, kLayoutWide><<<g, b, 0, stream>>>(s, f, st, bounce, cam);
            else
                extend_kernel<false, BATCH, PRIMARY, true, kLayoutWide><<<g, b, 0, stream>>>(s, f, st, bounce, cam);
        } else {
            if (count)
                extend_kernel<true, BATCH, PRIMARY, true, kLayoutQuant><<<g, b, 0, stream>>>(s, f, st, bounce, cam);
            else
                extend_kernel<false, BATCH, PRIMARY, true, kLayoutQuant><<<g, b, 0, stream>>>(s, f, st, bounce, cam);
        }
    };
    // batched paths make their camera rays in the launch from their sample ids,
    // never from a frame's camera (no PRIMARY variant)
    if constexpr (PRIMARY) {
        if (s.tlasNodes)
            twoLevel(std::false_type{});
        else
            oneLevel(std::false_type{});
    } else {
        if (f.batch && s.tlasNodes)
            twoLevel(std::true_type{});
        else if (f.batch)
            oneLevel(std::true_type{});
        else if (s.tlasNodes)
            twoLevel(std::false_type{});
        else
            oneLevel(std::false_type{});
    }
}

cudaError_t launch_extend(const SceneView& s, const FrameView& f, const Settings& st0, uint32_t bounce,
                          const LaunchShape& shape, cudaStream_t stream, const Camera* primary)
{
    Settings st = st0;
    st.refillBelow = shape.refillBelow;
    if (primary && bounce == 0 && (st.flags & TR_FLAG_REFERENCE_SAMPLING) == 0)
        launch_extend_variant<true>(s, f, st, bounce, *primary, shape, stream);
    else
        launch_extend_variant<false>(s, f, st, bounce, Camera{}, shape, stream);
    return cudaGetLastError();
}

cudaError_t launch_shade(const SceneView& s, const FrameView& f, const Settings& st, uint32_t bounce,
                         const LaunchShape& shape, cudaStream_t stream)
{
    const bool ref = (st.flags & TR_FLAG_REFERENCE_SAMPLING) != 0;
    const size_t smem = size_t(shape.shadeThreads) * kShadeStageBytes;
    if (f.batch && s.texSlots)
        shade_kernel<false, true, true><<<shape.shadeBlocks, shape.shadeThreads, smem, stream>>>(s, f, st, bounce);
    else if (f.batch)
        shade_kernel<false, true><<<shape.shadeBlocks, shape.shadeThreads, smem, stream>>>(s, f, st, bounce);
    else if (s.texSlots && ref)
        shade_kernel<true, false, true><<<shape.shadeBlocks, shape.shadeThreads, smem, stream>>>(s, f, st, bounce);
    else if (s.texSlots)
        shade_kernel<false, false, true><<<shape.shadeBlocks, shape.shadeThreads, smem, stream>>>(s, f, st, bounce);
    else if (ref)
        shade_kernel<true, false><<<shape.shadeBlocks, shape.shadeThreads, smem, stream>>>(s, f, st, bounce);
    else
        shade_kernel<false, false><<<shape.shadeBlocks, shape.shadeThreads, smem, stream>>>(s, f, st, bounce);
    return cudaGetLastError();
}

cudaError_t launch_connect(const SceneView& s0, const FrameView& f, const Settings& st0, uint32_t bounce,
                           const LaunchShape& shape, cudaStream_t stream)
{
    const SceneView s = traced(s0, st0);
    Settings st = st0;
    st.refillBelow = shape.refillBelow;
    const bool count = (st.flags & TR_FLAG_COUNT_TRAVERSAL) != 0;
    const uint32_t g = shape.connectBlocks;
    const uint32_t b = shape.traversalThreads;
    // one-level scenes: an instance per node layout
    auto oneLevel = [&](auto batchTag) {
        constexpr bool BATCH = decltype(batchTag)::value;
        if (s.quantNodes) {
            if (count)
                connect_kernel<true, BATCH, false, kLayoutQuant><<<g, b, 0, stream>>>(s, f, st, bounce);
            else
                connect_kernel<false, BATCH, false, kLayoutQuant><<<g, b, 0, stream>>>(s, f, st, bounce);
        } else {
            if (count)
                connect_kernel<true, BATCH, false, kLayoutWide><<<g, b, 0, stream>>>(s, f, st, bounce);
            else
                connect_kernel<false, BATCH, false, kLayoutWide><<<g, b, 0, stream>>>(s, f, st, bounce);
        }
    };
    auto twoLevel = [&](auto batchTag) {
        constexpr bool BATCH = decltype(batchTag)::value;
        if (!s.quantNodes) {
            if (count)
                connect_kernel<true, BATCH, true, kLayoutWide><<<g, b, 0, stream>>>(s, f, st, bounce);
            else
                connect_kernel<false, BATCH, true, kLayoutWide><<<g, b, 0, stream>>>(s, f, st, bounce);
        } else {
            if (count)
                connect_kernel<true, BATCH, true, kLayoutQuant><<<g, b, 0, stream>>>(s, f, st, bounce);
            else
                connect_kernel<false, BATCH, true, kLayoutQuant><<<g, b, 0, stream>>>(s, f, st, bounce);
        }
    };
    if (f.batch && s.tlasNodes)
        twoLevel(std::true_type{});
    else if (f.batch)
        oneLevel(std::true_type{});
    else if (s.tlasNodes)
        twoLevel(std::false_type{});
    else
        oneLevel(std::false_type{});
    return cudaGetLastError();
}

cudaError_t launch_advance(const FrameView& f, uint32_t samples, cudaStream_t stream)
{
    Settings st{};
    st.multiSample = samples;
    advance_kernel<<<1, 32, 0, stream>>>(f, st);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const FrameView& f, const Settings& st, cudaStream_t stream)
{
    const uint32_t wh = f.resX * f.resY;
    if (wh == 0)
        return cudaSuccess;
    finalize_kernel<<<(wh + 255u) / 256u, 256, 0, stream>>>(f, st);
    advance_kernel<<<1, 32, 0, stream>>>(f, st);
    return cudaGetLastError();
}

cudaError_t launch_adjoint(const SceneView& s0, const FrameView& f, const Camera& cam, const Settings& st,
                           const AdjointView& a, const LaunchShape& shape, cudaStream_t stream)
{
    const SceneView s = traced(s0, st);
    if (f.pathCount == 0)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(f.counters, 0, kCounterWords * sizeof(uint32_t), stream);
    if (e != cudaSuccess)
        return e;
    const size_t smem = size_t(kAdjointWarps) * a.materialCount * kGradSlots * sizeof(float);
    const bool useSmem = smem <= kAdjointSmemMax;
    int perSm = 0;
    e = useSmem ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, adjoint_shade_kernel<true>, kAdjointThreads,
                                                                smem)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, adjoint_shade_kernel<false>, kAdjointThreads,
                                                                0);
    if (e != cudaSuccess)
        return e;
    const uint32_t gradBlocks = shape.sms * uint32_t(perSm > 0 ? perSm : 1);
    // the replay's connect runs 128-thread blocks: as many threads as the forward connect grid
    const uint32_t connectBlocks128 = (shape.connectBlocks * shape.traversalThreads + 127u) / 128u;
    Settings fwd = st;
    fwd.flags &= ~uint32_t(TR_FLAG_COUNT_TRAVERSAL | TR_FLAG_WRITE_AOVS);
    fwd.refillBelow = shape.refillBelow;
    adjoint_generate_kernel<<<(f.pathCount + 255u) / 256u, 256, 0, stream>>>(f, cam, fwd, a);
    for (uint32_t bounce = 0; bounce < st.maxDepth; ++bounce) {
        if (s.tlasNodes && !s.quantNodes)
            extend_kernel<false, false, false, true, kLayoutWide>
                <<<shape.extendBlocks, shape.traversalThreads, 0, stream>>>(s, f, fwd, bounce, Camera{});
        else if (s.tlasNodes)
            extend_kernel<false, false, false, true, kLayoutQuant>
                <<<shape.extendBlocks, shape.traversalThreads, 0, stream>>>(s, f, fwd, bounce, Camera{});
        else if (s.quantNodes)
            extend_kernel<false, false, false, false, kLayoutQuant>
                <<<shape.extendBlocks, shape.traversalThreads, 0, stream>>>(s, f, fwd, bounce, Camera{});
        else
            extend_kernel<false, false, false, false, kLayoutWide>
                <<<shape.extendBlocks, shape.traversalThreads, 0, stream>>>(s, f, fwd, bounce, Camera{});
        if (bounce > 0) {
            if (useSmem)
                ext_grad_kernel<true><<<gradBlocks, kAdjointThreads, smem, stream>>>(s, f, bounce, a);
            else
                ext_grad_kernel<false><<<gradBlocks, kAdjointThreads, 0, stream>>>(s, f, bounce, a);
        }
        if (useSmem)
            adjoint_shade_kernel<true><<<gradBlocks, kAdjointThreads, smem, stream>>>(s, f, fwd, bounce, a);
        else
            adjoint_shade_kernel<false><<<gradBlocks, kAdjointThreads, 0, stream>>>(s, f, fwd, bounce, a);
        if (s.tlasNodes)
            adjoint_connect_kernel<true><<<connectBlocks128, 128, 0, stream>>>(s, f, fwd, bounce, a);
        else
            adjoint_connect_kernel<false><<<connectBlocks128, 128, 0, stream>>>(s, f, fwd, bounce, a);
        if (useSmem)
            nee_grad_kernel<true><<<gradBlocks, kAdjointThreads, smem, stream>>>(s, f, bounce, a);
        else
            nee_grad_kernel<false><<<gradBlocks, kAdjointThreads, 0, stream>>>(s, f, bounce, a);
    }
    return cudaGetLastError();
}

cudaError_t launch_debug_bounce(const SceneView& s0, const FrameView& f, const Camera& cam, const Settings& st,
                                uint32_t bounce, const LaunchShape& shape, cudaStream_t stream)
{
    const SceneView s = traced(s0, st);
    const uint32_t blocks = shape.sms * 8u;
    debug_extend_kernel<<<blocks, 128, 0, stream>>>(s, f, cam, st, bounce);
    debug_shade_kernel<<<blocks, 128, 0, stream>>>(s, f, cam, st, bounce);
    return cudaGetLastError();
}

cudaError_t launch_pick_ray(const SceneView& s, const Camera& cam, const Settings& st, uint32_t resX, uint32_t resY,
                            int x, int y, float* result, uint32_t* errorFlag, cudaStream_t stream)
{
    pick_ray_kernel<<<1, 32, 0, stream>>>(traced(s, st), cam, st, resX, resY, x, y, result, errorFlag);
    return cudaGetLastError();
}

cudaError_t launch_sort_hits(const SceneView& s, const FrameView& f, const SortView& sv, uint32_t bounce,
                             const LaunchShape& shape, cudaStream_t stream)
{
    const uint32_t blocks = shape.sms * 4u;
    sort_histogram_kernel<<<blocks, 256, 0, stream>>>(s, f, sv, bounce);
    sort_scan_kernel<<<1, 1024, 0, stream>>>(sv);
    sort_scatter_kernel<<<blocks, 256, 0, stream>>>(f, sv, bounce);
    return cudaGetLastError();
}

cudaError_t launch_batch_plan(BatchState* state, uint32_t pool, uint32_t end, uint32_t limit, uint32_t* errorFlag,
                              cudaGraphConditionalHandle loop, bool useLoop, cudaStream_t stream)
{
    batch_plan_kernel<<<1, 32, 0, stream>>>(state, pool, end, limit, errorFlag, loop, useLoop ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_batch_finalize(const FrameView& f, uint32_t pixelBegin, uint32_t pixelEnd, cudaStream_t stream)
{
    if (pixelEnd <= pixelBegin)
        return cudaSuccess;
    batch_finalize_kernel<<<(pixelEnd - pixelBegin + 255u) / 256u, 256, 0, stream>>>(f, pixelBegin, pixelEnd);
    return cudaGetLastError();
}

namespace {
// Resident blocks per SM of `kernel` at `threads` per block (4 when the query fails).
template <class Kernel>
uint32_t resident(Kernel kernel, uint32_t threads, size_t smem)
{
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, int(threads), smem);
    return uint32_t(perSm > 0 ? perSm : 4);
}

// Block sizes the traversal and shade kernels take: their register budgets are
// set for blocks of at most 128 threads.
bool valid_threads(uint32_t t) { return t == 64u || t == 128u; }

// Grids of a shape for its block sizes: the persistent traversal kernels at
// their occupancy limit, shade capped at shadeWaves waves of resident blocks.
void size_grids(LaunchShape& shape, uint32_t capacity)
{
    shape.extendPerSm = resident(extend_kernel<false, false, false, false, kLayoutWide>, shape.traversalThreads, 0);
    shape.connectPerSm = resident(connect_kernel<false, false, false, kLayoutWide>, shape.traversalThreads, 0);
    shape.extendBlocks = shape.sms * shape.extendPerSm;
    shape.connectBlocks = shape.sms * shape.connectPerSm;
    const uint32_t maxShade = shape.sms *
                              resident(shade_kernel<false, false>, shape.shadeThreads,
                                       size_t(shape.shadeThreads) * kShadeStageBytes) *
                              shape.shadeWaves;
    const uint32_t need = (capacity + shape.shadeThreads - 1u) / shape.shadeThreads;
    shape.shadeBlocks = need < maxShade ? (need > 0 ? need : 1u) : maxShade;
}
} // namespace

LaunchShape default_launch_shape(int device, uint32_t capacity)
{
    LaunchShape shape;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    shape.sms = uint32_t(sms > 0 ? sms : 1);
    shape.refillBelow = kRefillBelow;
    shape.shadeWaves = 4;
    shape.traversalThreads = 128;
    shape.shadeThreads = 128;
    size_grids(shape, capacity);
    return shape;
}

LaunchShape tuned_launch_shape(int device, uint32_t capacity, const tr_tuning& t)
{
    LaunchShape shape = default_launch_shape(device, capacity);
    if (t.refill_below >= 1 && t.refill_below <= 32)
        shape.refillBelow = t.refill_below;
    if (t.shade_waves >= 1 && t.shade_waves <= 64)
        shape.shadeWaves = t.shade_waves;
    if (valid_threads(t.traversal_threads))
        shape.traversalThreads = t.traversal_threads;
    if (valid_threads(t.shade_threads))
        shape.shadeThreads = t.shade_threads;
    size_grids(shape, capacity);
    if (t.extend_blocks_per_sm >= 1 && t.extend_blocks_per_sm <= shape.extendPerSm)
        shape.extendBlocks = shape.sms * t.extend_blocks_per_sm;
    if (t.connect_blocks_per_sm >= 1 && t.connect_blocks_per_sm <= shape.connectPerSm)
        shape.connectBlocks = shape.sms * t.connect_blocks_per_sm;
    shape.sortHits = t.sort_hits ? 1u : 0u;
    return shape;
}

} // namespace tr
