"""Differentiable rendering: a libtorch torch::autograd::Function
(torch_op/render_op.cpp) whose forward renders through the C ABI and whose
backward runs the path-replay adjoint kernel (tr_adjoint_frame).

The extension is compiled on first use into trayracer_gb300/_build/torch_op
(it links libtrayracer.so; no CUDA code of its own).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .renderer import DeviceRenderer, KernelSettings
from .scenes import MATERIAL_DTYPE, Scene

PKG = Path(__file__).resolve().parent
_op = None

PARAM_NAMES = ["base_r", "base_g", "base_b", "roughness", "metallic", "specular", "emission_r", "emission_g",
               "emission_b"]


def load_op():
    global _op
    if _op is None:
        from . import build as tb
        from torch.utils.cpp_extension import load

        tb.build()
        bdir = PKG / "_build" / "torch_op"
        bdir.mkdir(parents=True, exist_ok=True)
        _op = load(
            name="trayracer_render_op",
            sources=[str(PKG / "torch_op" / "render_op.cpp")],
            extra_cflags=["-O2"],
            extra_ldflags=[f"-L{PKG}", "-ltrayracer", f"-Wl,-rpath,{PKG}"],
            build_directory=str(bdir),
            with_cuda=True,
            verbose=False,
        )
    return _op


def material_params(materials: np.ndarray) -> np.ndarray:
    """(M, 9) float32: base colour rgb, roughness, metallic, specular, emission rgb."""
    m = np.asarray(materials, MATERIAL_DTYPE)
    p = np.zeros((m.shape[0], 9), np.float32)
    p[:, 0:3] = m["diffuse"]
    p[:, 3] = m["roughness"]
    p[:, 4] = m["metallic"]
    p[:, 5] = m["specular"]
    p[:, 6:9] = m["emissive"]
    return p


class DifferentiableRenderer:
    """Renders `scene` with all samples in one wavefront frame; render(params)
    is differentiable with respect to the (materials, 9) parameter tensor."""

    def __init__(self, scene: Scene, spp: int, max_depth: int, seed: int = 1, device: int = 0,
                 max_color: float = 1e30):
        import torch

        self.scene = scene
        self.renderer = DeviceRenderer(device)
        self.renderer.UpdateScene(scene)
        self.renderer.SetCamera(scene.camera)
        self.renderer.Resize((scene.width, scene.height))
        self.settings = KernelSettings(multiSample=spp, maxDepth=max_depth, seed=seed, rrStart=1 << 30,
                                       maxColor=max_color)
        self.renderer.SetSettings(self.settings)
        self.base = torch.from_numpy(np.ascontiguousarray(scene.materials, MATERIAL_DTYPE).view(np.uint8).copy())
        self.op = load_op()

    def initial_params(self):
        import torch

        return torch.from_numpy(material_params(self.scene.materials))

    def render(self, params):
        return self.op.render(params, self.base, int(self.renderer.handle.value))

    def close(self):
        self.renderer.close()
