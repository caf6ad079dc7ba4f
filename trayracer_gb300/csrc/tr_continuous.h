// The continuous wavefront: a pool of path slots kept full from a device
// sample cursor (used by batched rendering, tr_batch_*, and by
// tr_render_samples for one scene). No counterpart in the reference, whose
// DeviceRenderer renders frame by frame with a host bounce loop
// (Tracer/Renderer/DeviceRenderer.cpp:97-133).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "tr_device.h"
#include "tr_kernels.h"

namespace tr {

// One round: items whose samples share one per-sample radiance buffer.
struct ContinuousRound {
    FrameView frame;      // pool queues, per-sample radiance, the round's items and BatchState
    uint32_t samples;     // sample ids [0, samples)
    uint32_t pixelBegin;  // the round's pixels in the accumulator
    uint32_t pixelEnd;
};

// What the launches share: scene, settings, launch shapes, path slots, and the
// side stream with its fork / join events on which a captured iteration traces
// the last iteration's shadow rays beside its extend.
struct ContinuousLaunch {
    SceneView scene;
    Settings settings;
    LaunchShape shape;
    uint32_t pool;
    cudaStream_t side;
    cudaEvent_t fork;
    cudaEvent_t join;
};

// Device time per stage of an eager run, summed over its iterations (CUDA
// events around each stage on the launch stream; the stages run in sequence).
struct StageTimes {
    float plan = 0.f;     // plan kernels (totals, queue hand-over, new samples taken)
    float connect = 0.f;  // shadow rays
    float extend = 0.f;   // carried paths and the camera rays of new samples
    float shade = 0.f;
    float end = 0.f;      // round starts, finalize and the sample count advance
};

// One iteration of a round: plan, connect of the last iteration's shadow rays
// and extend (carried paths + new samples), shade. With `overlap`, connect
// runs on the side stream beside extend: connect reads the shadow queue and
// adds to the radiance of paths in flight, extend reads the extend queue and
// starts new samples, so they share nothing; shade (which rewrites the shadow
// queue and adds emission to the same radiance) waits for both. Not with a
// sky, whose misses extend adds to the radiance of carried paths.
// `marks` (optional, without overlap): four events recorded after plan,
// connect, extend and shade.
cudaError_t enqueue_continuous_iteration(const ContinuousLaunch& L, const ContinuousRound& r,
                                         cudaGraphConditionalHandle loop, bool useLoop, cudaStream_t s,
                                         bool overlap, const cudaEvent_t* marks = nullptr);

// A graph of all rounds in order: per round its start, a while loop over its
// iterations (condition set by the plan kernel on the device) and its
// finalize; then `advance` added to the device sample count (0: none).
// Captured on `s`, which must not be capturing and must be idle.
cudaError_t capture_continuous(const ContinuousLaunch& L, const std::vector<ContinuousRound>& rounds,
                               uint32_t advance, cudaStream_t s, cudaGraph_t* out);

// The same launches from a host loop that reads each round's queue length
// back after every iteration (no graph), stages in sequence. With `times`, the
// device time of each stage is summed into it (the call then returns with the
// stream idle).
cudaError_t run_continuous_eager(const ContinuousLaunch& L, const std::vector<ContinuousRound>& rounds,
                                 uint32_t advance, cudaStream_t s, StageTimes* times = nullptr);

} // namespace tr
