"""The other render modes (RenderModes other than PathTracing: ambient occlusion,
normals, tangents, IDs, material properties, texture coordinates, wireframe, depth)
against images the reference's own raygen programs and shade kernels made
(tests/golden/ref_debug_modes.npz, tests/golden/make_golden.py debug_modes) on the
two-level Cornell box, one frame at one sample per pixel in reference sampling."""
from pathlib import Path

import numpy as np
import pytest

import trayracer_gb300 as tr
from trayracer_gb300._abi import TR_FLAG_REFERENCE_DRAW_RTL
from trayracer_gb300.renderer import KernelSettings, RenderModes

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_debug_modes.npz"

# modes whose value depends only on the primary hit: per-pixel agreement within
# 1e-5 relative (the GPU contracts multiply-adds); the sampled modes (occlusion rays
# from sincosf directions, the wireframe's jittered second ray) may flip a hit on a
# last-bit difference at an edge
SAMPLED = {RenderModes.AmbientOcclusion, RenderModes.AmbientOcclusionShading, RenderModes.Wireframe}


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def renderer(golden):
    w, h = int(golden["width"]), int(golden["height"])
    scene = tr.instanced_cornell(width=w, height=h)
    assert scene.digest() == str(golden["digest"]), "scene generator drifted from the fixture"
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene)
    r.SetCamera(scene.camera)
    r.Resize((w, h))
    yield r
    r.close()


def _settings(golden):
    return KernelSettings(multiSample=1, maxDepth=2, seed=int(golden["seed"]), rrStart=1,
                          aoDist=float(golden["ao_dist"]), zDepthMax=float(golden["z_depth_max"]),
                          flags=tr.TR_FLAG_REFERENCE_SAMPLING | TR_FLAG_REFERENCE_DRAW_RTL)


@pytest.mark.parametrize("mode,flags", [tuple(int(v) for v in m) for m in np.load(GOLDEN)["modes"]])
def test_render_mode_matches_reference(golden, renderer, mode, flags):
    want = golden[f"mode_{mode}_{flags}"]
    renderer.Reset()
    renderer.RenderFrame(_settings(golden), RenderModes(mode), flags)
    got = renderer.Accumulator().reshape(-1, 4)
    ok = np.isclose(got[:, :3], want[:, :3], rtol=1e-5, atol=1e-6).all(1)
    np.testing.assert_array_equal(got[:, 3], want[:, 3])  # sample counts
    if RenderModes(mode) in SAMPLED:
        assert ok.mean() >= 0.97, ok.mean()
        assert abs(got[:, :3].mean() - want[:, :3].mean()) <= 0.01 * max(1e-3, want[:, :3].mean())
    else:
        assert ok.mean() >= 0.995, ok.mean()


def test_modes_switch_back_to_path_tracing(golden, renderer):
    st = _settings(golden)
    renderer.Reset()
    renderer.RenderFrame(st, RenderModes.PathTracing)
    a = renderer.Accumulator().copy()
    renderer.RenderFrame(st, RenderModes.ShadingNormal)  # resets, one frame of normals
    assert renderer.SampleCount() == 1
    renderer.RenderFrame(st, RenderModes.PathTracing)  # resets again
    np.testing.assert_array_equal(renderer.Accumulator(), a)
    with pytest.raises(tr.TracerError):
        renderer.RenderFrame(st, 13)
    # the per-stage entries drive the path-tracing mode only
    renderer.RenderFrame(st, RenderModes.ZDepth)
    with pytest.raises(tr.TracerError):
        renderer.Extend(0)
    renderer.RenderFrame(st, RenderModes.PathTracing)
