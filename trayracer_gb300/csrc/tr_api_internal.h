// Read access to a context's scene, camera and settings for entry points that
// live outside tr_api.cpp, and the ABI conversions they share. None of these
// functions allocates device memory.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "tr_device.h"

namespace tr {

struct ContextViews {
    int device;
    cudaStream_t stream;     // the context's own stream
    SceneView scene;
    Camera camera;
    Settings settings;
    uint32_t width;
    uint32_t height;
};

// TR_OK with the views of a context that has a scene, a camera and a resolution.
tr_status context_views(void* ctx, ContextViews* out);
// Records msg as the context's last error and returns st.
tr_status context_fail(void* ctx, tr_status st, const std::string& msg);

// Checked conversions of the ABI camera and settings (false + *err when invalid).
bool convert_camera(const tr_camera& cam, Camera* out, std::string* err);
bool convert_settings(const tr_kernel_settings& s, Settings* out, std::string* err);

} // namespace tr
