// libtorch autograd function over the C ABI: forward renders the image for a
// table of material parameters, backward runs the path-replay adjoint
// (tr_adjoint_frame) and returns d loss / d parameters.
//
// Parameters per material (9 floats): base colour r, g, b, roughness,
// metallic, specular, emission r, g, b. The remaining material properties
// come from the scene's material table (`base`, tr_material_desc records).
#include <torch/extension.h>

#include <ATen/cuda/CUDAContext.h>
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/trayracer.h"

namespace {

void check(tr_status st, void* ctx, const char* what)
{
    if (st != TR_OK)
        throw std::runtime_error(std::string(what) + ": " + tr_status_string(st) + ": " + tr_last_error(ctx));
}

class RenderFunction : public torch::autograd::Function<RenderFunction> {
public:
    static torch::Tensor forward(torch::autograd::AutogradContext* actx, torch::Tensor params, torch::Tensor base,
                                 int64_t handle)
    {
        void* ctx = reinterpret_cast<void*>(handle);
        const int64_t m = params.size(0);
        TORCH_CHECK(params.dim() == 2 && params.size(1) == 9, "params must be (materials, 9)");
        TORCH_CHECK(base.scalar_type() == torch::kUInt8 && base.numel() == m * int64_t(sizeof(tr_material_desc)),
                    "base must hold one tr_material_desc per material");
        const torch::Tensor p = params.detach().to(torch::kCPU, torch::kFloat32).contiguous();
        const torch::Tensor b = base.to(torch::kCPU).contiguous();
        std::vector<tr_material_desc> mats(static_cast<size_t>(m));
        std::memcpy(mats.data(), b.data_ptr(), mats.size() * sizeof(tr_material_desc));
        const float* pp = p.data_ptr<float>();
        for (int64_t i = 0; i < m; ++i) {
            const float* q = pp + 9 * i;
            tr_material_desc& d = mats[size_t(i)];
            d.diffuse[0] = q[0];
            d.diffuse[1] = q[1];
            d.diffuse[2] = q[2];
            d.roughness = q[3];
            d.metallic = q[4];
            d.specular = q[5];
            d.emissive[0] = q[6];
            d.emissive[1] = q[7];
            d.emissive[2] = q[8];
        }
        check(tr_update_materials(ctx, mats.data(), uint32_t(m)), ctx, "tr_update_materials");
        cudaStream_t stream = at::cuda::getCurrentCUDAStream();
        // one frame holds every sample: the adjoint replays the paths of the last frame
        check(tr_render_frame(ctx, stream, 1), ctx, "tr_render_frame");
        tr_buffers buf{};
        check(tr_get_buffers(ctx, &buf), ctx, "tr_get_buffers");
        auto img = torch::empty({int64_t(buf.height), int64_t(buf.width), 4},
                                torch::TensorOptions().dtype(torch::kFloat32).device(torch::kCUDA));
        const size_t bytes = size_t(buf.width) * buf.height * 16;
        TORCH_CHECK(cudaMemcpyAsync(img.data_ptr(), buf.colors, bytes, cudaMemcpyDeviceToDevice, stream) ==
                        cudaSuccess,
                    "image copy failed");
        tr_statistics stats{};
        actx->saved_data["handle"] = handle;
        actx->saved_data["materials"] = m;
        actx->saved_data["samples"] = int64_t(buf.capacity / (uint64_t(buf.width) * buf.height));
        actx->saved_data["device"] = params.device().str();
        (void)stats;
        return img;
    }

    static torch::autograd::tensor_list backward(torch::autograd::AutogradContext* actx,
                                                 torch::autograd::tensor_list grads)
    {
        void* ctx = reinterpret_cast<void*>(actx->saved_data["handle"].toInt());
        const int64_t m = actx->saved_data["materials"].toInt();
        const int64_t samples = actx->saved_data["samples"].toInt();
        const torch::Tensor g = grads[0].to(torch::kCUDA, torch::kFloat32).contiguous();
        auto out = torch::zeros({m, 9}, torch::TensorOptions().dtype(torch::kFloat32).device(torch::kCUDA));
        cudaStream_t stream = at::cuda::getCurrentCUDAStream();
        check(tr_adjoint_frame(ctx, stream, g.data_ptr<float>(), 1.0f / float(samples), out.data_ptr<float>()), ctx,
              "tr_adjoint_frame");
        const torch::Device dev(actx->saved_data["device"].toStringRef());
        return {out.to(dev), torch::Tensor(), torch::Tensor()};
    }
};

torch::Tensor render(torch::Tensor params, torch::Tensor base, int64_t handle)
{
    return RenderFunction::apply(params, base, handle);
}

} // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m)
{
    m.def("render", &render, "Render the image for material parameters (differentiable: path-replay adjoint)");
}
