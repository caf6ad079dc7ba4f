// The continuous wavefront's launch sequence, graph and host loop (see
// tr_continuous.h).
#include "tr_continuous.h"

namespace tr {
namespace {

// A round ends after at most samples * max_depth iterations (every path ends
// within max_depth of them); the plan kernel stops the loop there with the
// error word set should the counts ever say otherwise.
uint32_t iteration_limit(const ContinuousRound& r, const Settings& st)
{
    const uint64_t bound = uint64_t(r.samples) * st.maxDepth + 4u;
    return bound < 0xffffffffull ? uint32_t(bound) : 0xffffffffu;
}

cudaError_t enqueue_round_start(const ContinuousRound& r, cudaStream_t s)
{
    return cudaMemsetAsync(r.frame.batch, 0, sizeof(BatchState), s);
}

cudaError_t enqueue_round_end(const ContinuousRound& r, cudaStream_t s)
{
    return launch_batch_finalize(r.frame, r.pixelBegin, r.pixelEnd, s);
}

// Captures body() on s into `into` after `deps`; *tail (optional) gets the
// last node captured.
template <class Body>
cudaError_t capture_into(cudaStream_t s, cudaGraph_t into, const cudaGraphNode_t* deps, size_t nDeps, Body&& body,
                         cudaGraphNode_t* tail)
{
    cudaError_t e = cudaStreamBeginCaptureToGraph(s, into, deps, nullptr, nDeps, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return e;
    e = body();
    if (e == cudaSuccess && tail) {
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* d = nullptr;
        size_t n = 0;
        e = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &d, nullptr, &n);
        if (e == cudaSuccess)
            *tail = n ? d[n - 1] : nullptr;
        if (e == cudaSuccess && !*tail)
            e = cudaErrorStreamCaptureInvalidated;
    }
    cudaGraph_t out = into;
    const cudaError_t ee = cudaStreamEndCapture(s, &out);
    return e != cudaSuccess ? e : ee;
}

// Events of a timed eager run.
struct TimingEvents {
    cudaEvent_t ev[5] = {};
    cudaError_t create()
    {
        for (cudaEvent_t& e : ev) {
            const cudaError_t x = cudaEventCreate(&e);
            if (x != cudaSuccess)
                return x;
        }
        return cudaSuccess;
    }
    ~TimingEvents()
    {
        for (cudaEvent_t e : ev)
            if (e)
                cudaEventDestroy(e);
    }
};

// Adds the time from event a to event b (both complete) to *acc.
cudaError_t add_elapsed(cudaEvent_t a, cudaEvent_t b, float* acc)
{
    float ms = 0.f;
    const cudaError_t e = cudaEventElapsedTime(&ms, a, b);
    if (e == cudaSuccess)
        *acc += ms;
    return e;
}

} // namespace

cudaError_t enqueue_continuous_iteration(const ContinuousLaunch& L, const ContinuousRound& r,
                                         cudaGraphConditionalHandle loop, bool useLoop, cudaStream_t s, bool overlap,
                                         const cudaEvent_t* marks)
{
    const FrameView& f = r.frame;
    cudaError_t e = launch_batch_plan(f.batch, L.pool, r.samples, iteration_limit(r, L.settings), f.errorFlag, loop,
                                      useLoop, s);
    // with a sky, extend adds the sky to the radiance of a carried path that
    // misses, which connect may be adding to at the same time
    if (overlap && !L.scene.sky.enabled) {
        marks = nullptr;
        if (e == cudaSuccess)
            e = cudaEventRecord(L.fork, s);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(L.side, L.fork, 0);
        if (e == cudaSuccess)
            e = launch_connect(L.scene, f, L.settings, 0u, L.shape, L.side);
        if (e == cudaSuccess)
            e = cudaEventRecord(L.join, L.side);
        if (e == cudaSuccess)
            e = launch_extend(L.scene, f, L.settings, 0u, L.shape, s, nullptr);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(s, L.join, 0);
    } else {
        if (e == cudaSuccess && marks)
            e = cudaEventRecord(marks[0], s);
        if (e == cudaSuccess)
            e = launch_connect(L.scene, f, L.settings, 0u, L.shape, s);
        if (e == cudaSuccess && marks)
            e = cudaEventRecord(marks[1], s);
        if (e == cudaSuccess)
            e = launch_extend(L.scene, f, L.settings, 0u, L.shape, s, nullptr);
        if (e == cudaSuccess && marks)
            e = cudaEventRecord(marks[2], s);
    }
    if (e == cudaSuccess)
        e = launch_shade(L.scene, f, L.settings, 0u, L.shape, s);
    if (e == cudaSuccess && marks)
        e = cudaEventRecord(marks[3], s);
    return e;
}

cudaError_t capture_continuous(const ContinuousLaunch& L, const std::vector<ContinuousRound>& rounds,
                               uint32_t advance, cudaStream_t s, cudaGraph_t* out)
{
    *out = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess)
        return e;
    cudaGraphNode_t last = nullptr;
    for (size_t k = 0; e == cudaSuccess && k < rounds.size(); ++k) {
        const ContinuousRound& r = rounds[k];
        cudaGraphNode_t start = nullptr;
        e = capture_into(s, g, last ? &last : nullptr, last ? 1 : 0, [&]() { return enqueue_round_start(r, s); },
                         &start);
        cudaGraphConditionalHandle loop{};
        if (e == cudaSuccess)
            e = cudaGraphConditionalHandleCreate(&loop, g, 1u, cudaGraphCondAssignDefault);
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = loop;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t whileNode = nullptr;
        if (e == cudaSuccess)
            e = cudaGraphAddNode(&whileNode, g, &start, nullptr, 1, &cp);
        if (e == cudaSuccess)
            e = capture_into(s, cp.conditional.phGraph_out[0], nullptr, 0,
                             [&]() { return enqueue_continuous_iteration(L, r, loop, true, s, true); }, nullptr);
        if (e == cudaSuccess)
            e = capture_into(
                s, g, &whileNode, 1,
                [&]() {
                    cudaError_t x = enqueue_round_end(r, s);
                    if (x == cudaSuccess && advance && k + 1 == rounds.size())
                        x = launch_advance(r.frame, advance, s);
                    return x;
                },
                &last);
    }
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return e;
    }
    *out = g;
    return cudaSuccess;
}

cudaError_t run_continuous_eager(const ContinuousLaunch& L, const std::vector<ContinuousRound>& rounds,
                                 uint32_t advance, cudaStream_t s, StageTimes* times)
{
    TimingEvents t;
    cudaError_t e = times ? t.create() : cudaSuccess;
    // t.ev[0] before a stage group, t.ev[1..4] the marks after plan, connect, extend, shade
    const auto mark = [&](int i) { return times ? cudaEventRecord(t.ev[i], s) : cudaSuccess; };
    const auto end_group = [&]() {
        cudaError_t x = mark(1);
        if (x == cudaSuccess && times)
            x = cudaEventSynchronize(t.ev[1]);
        if (x == cudaSuccess && times)
            x = add_elapsed(t.ev[0], t.ev[1], &times->end);
        return x;
    };
    for (size_t k = 0; e == cudaSuccess && k < rounds.size(); ++k) {
        const ContinuousRound& r = rounds[k];
        e = mark(0);
        if (e == cudaSuccess)
            e = enqueue_round_start(r, s);
        if (e == cudaSuccess)
            e = end_group();
        while (e == cudaSuccess) {
            e = mark(0);
            if (e == cudaSuccess)
                e = enqueue_continuous_iteration(L, r, cudaGraphConditionalHandle{}, false, s, false,
                                                 times ? t.ev + 1 : nullptr);
            uint32_t queue = 0;
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(&queue, &r.frame.batch->queue, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(s);
            if (e == cudaSuccess && times) {
                e = add_elapsed(t.ev[0], t.ev[1], &times->plan);
                if (e == cudaSuccess)
                    e = add_elapsed(t.ev[1], t.ev[2], &times->connect);
                if (e == cudaSuccess)
                    e = add_elapsed(t.ev[2], t.ev[3], &times->extend);
                if (e == cudaSuccess)
                    e = add_elapsed(t.ev[3], t.ev[4], &times->shade);
            }
            if (e != cudaSuccess || queue == 0)
                break;
        }
        if (e == cudaSuccess)
            e = mark(0);
        if (e == cudaSuccess)
            e = enqueue_round_end(r, s);
        if (e == cudaSuccess && advance && k + 1 == rounds.size())
            e = launch_advance(r.frame, advance, s);
        if (e == cudaSuccess)
            e = end_group();
    }
    return e;
}

} // namespace tr
