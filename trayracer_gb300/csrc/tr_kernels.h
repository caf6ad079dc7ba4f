// Host-side launchers of the wavefront kernels.
#pragma once

#include <cuda_runtime.h>

#include "tr_device.h"
#include "../../include/trayracer.h"

namespace tr {

// Grid sizes: extend/connect are persistent (resident blocks per SM x SMs,
// warps fetch 32 rays at a time from a device cursor); shade is a
// warp-strided grid capped at a few waves.
struct LaunchShape {
    uint32_t extendBlocks = 0;
    uint32_t connectBlocks = 0;
    uint32_t shadeBlocks = 0;
    uint32_t sms = 0;
    uint32_t refillBelow = 10;   // lane refill threshold of the persistent traversal warps
    uint32_t extendPerSm = 0;    // resident extend / connect blocks per SM (occupancy limit by default)
    uint32_t connectPerSm = 0;
    uint32_t shadeWaves = 4;     // shade grid cap, in waves of resident blocks
    uint32_t sortHits = 0;       // 1: counting sort of each bounce's hit queue by material before shade
    uint32_t traversalThreads = 128;  // block size of the extend and connect launches (64 or 128)
    uint32_t shadeThreads = 128;      // block size of the shade launches (64 or 128)
};

LaunchShape default_launch_shape(int device, uint32_t capacity);
// The default shape with the tunable fields of t applied (zero fields keep the default).
LaunchShape tuned_launch_shape(int device, uint32_t capacity, const tr_tuning& t);

cudaError_t launch_generate(const FrameView& f, const Camera& cam, const Settings& st, cudaStream_t stream);
// primary != nullptr at bounce 0 (default sampling mode): the camera rays are
// computed inside the extend launch and no generate launch is needed.
cudaError_t launch_extend(const SceneView& s, const FrameView& f, const Settings& st, uint32_t bounce,
                          const LaunchShape& shape, cudaStream_t stream, const Camera* primary = nullptr);
cudaError_t launch_shade(const SceneView& s, const FrameView& f, const Settings& st, uint32_t bounce,
                         const LaunchShape& shape, cudaStream_t stream);
cudaError_t launch_connect(const SceneView& s, const FrameView& f, const Settings& st, uint32_t bounce,
                           const LaunchShape& shape, cudaStream_t stream);
cudaError_t launch_finalize(const FrameView& f, const Settings& st, cudaStream_t stream);
// Adds `samples` to the frame's device sample count.
cudaError_t launch_advance(const FrameView& f, uint32_t samples, cudaStream_t stream);
// One bounce of a debug render mode (Settings::renderMode != path tracing):
// closest hit of every ray of queue state[bounce & 1], then the mode's shade.
cudaError_t launch_debug_bounce(const SceneView& s, const FrameView& f, const Camera& cam, const Settings& st,
                                uint32_t bounce, const LaunchShape& shape, cudaStream_t stream);
// RayPick: one camera ray through pixel (x, resY - y), closest hit; result holds
// 9 words laid out as tr_ray_pick_result.
cudaError_t launch_pick_ray(const SceneView& s, const Camera& cam, const Settings& st, uint32_t resX, uint32_t resY,
                            int x, int y, float* result, uint32_t* errorFlag, cudaStream_t stream);
// Counting sort of the bounce's hit queue by material into sv.order (shade
// reads the queue through it when FrameView::hitOrder = sv.order).
cudaError_t launch_sort_hits(const SceneView& s, const FrameView& f, const SortView& sv, uint32_t bounce,
                             const LaunchShape& shape, cudaStream_t stream);
// Batched rendering: the plan of one iteration of the continuous wavefront
// (with useLoop, it sets the conditional of the graph's while loop: 1 while
// there are rays to trace; a round stops after `limit` iterations with the
// error word set), and the accumulator and colors of a round's
// pixels [pixelBegin, pixelEnd) from its per-sample radiance.
cudaError_t launch_batch_plan(BatchState* state, uint32_t pool, uint32_t end, uint32_t limit, uint32_t* errorFlag,
                              cudaGraphConditionalHandle loop, bool useLoop, cudaStream_t stream);
cudaError_t launch_batch_finalize(const FrameView& f, uint32_t pixelBegin, uint32_t pixelEnd, cudaStream_t stream);
// Path-replay adjoint of the frame `f` (its per-path radiance and sample
// count are the forward frame's; its queues are overwritten, its counters
// are the adjoint's own).
cudaError_t launch_adjoint(const SceneView& s, const FrameView& f, const Camera& cam, const Settings& st,
                           const AdjointView& a, const LaunchShape& shape, cudaStream_t stream);

} // namespace tr
