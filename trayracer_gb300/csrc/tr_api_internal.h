// Read access to a context's scene, camera and settings for entry points that
// live outside tr_api.cpp, and the ABI conversions they share. None of these
// functions allocates device memory.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "tr_device.h"
#include "tr_kernels.h"

namespace tr {

struct ContextViews {
    int device;
    cudaStream_t stream;     // the context's own stream
    SceneView scene;
    Camera camera;
    Settings settings;
    uint32_t width;
    uint32_t height;
    uint32_t renderMode;     // RenderModes value set by tr_set_render_mode
};

// Device words of a frame that tr_get_statistics reads.
struct FrameWords {
    uint32_t* counters;            // kCounterWords
    uint32_t* sampleCount;
    uint32_t* errorFlag;
    unsigned long long* traversal; // 4 counters
};

// A texture as the kernels sample it (RGBA binary16, bilinear, wrap,
// normalised coordinates): its CUDA array (set as soon as allocated, so that a
// caller can free it on an error) and texture object.
cudaError_t create_texture(const tr_texture_desc& t, cudaArray_t* arr, cudaTextureObject_t* obj);

// TR_OK with the views of a context that has a scene, a camera and a resolution.
tr_status context_views(void* ctx, ContextViews* out);
// The context's launch shape (its tuning applied) for `capacity` paths in
// flight, without the hit sort; cached in the context until the tuning or the
// capacity changes.
tr_status context_launch_shape(void* ctx, uint32_t capacity, LaunchShape* out);
// Marks the last frame of the context as one rendered by
// tr_render_frame_noalloc with `paths` paths in flight: tr_get_statistics then
// reads that frame's words from the no-allocation scratch.
void context_note_noalloc_frame(void* ctx, uint32_t paths);
// Device words of the no-allocation frame on `device` (its scratch array).
tr_status noalloc_frame_words(int device, FrameWords* out, std::string& err);
// Records msg as the context's last error and returns st.
tr_status context_fail(void* ctx, tr_status st, const std::string& msg);

// Checked conversions of the ABI camera and settings (false + *err when invalid).
bool convert_camera(const tr_camera& cam, Camera* out, std::string* err);
bool convert_settings(const tr_kernel_settings& s, Settings* out, std::string* err);

} // namespace tr
