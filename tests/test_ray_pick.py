"""Ray pick (DeviceRenderer::PickRay, DeviceRenderer.cpp:71-92, RayPick raygen optix.cu:345-377)
against results of the reference's own raygen compiled as host C++ (tests/golden/ref_ray_pick.npz,
made by tests/golden/make_golden.py ray_picks): the oracle on the CPU, the library on the GPU."""
from pathlib import Path

import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle, Reference, reference_available
from trayracer_gb300._abi import TR_FLAG_REFERENCE_DRAW_RTL
from trayracer_gb300.renderer import KernelSettings
from trayracer_gb300.scenes import CameraSpec

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_ray_pick.npz"
SCENES = {
    "cornell": lambda: tr.cornell_box(width=40, height=30),
    "instanced_cornell": lambda: tr.instanced_cornell(width=40, height=30),
    "heightfield_lens": lambda: tr.heightfield(n=16, width=32, height=32),
}
MISS = 0xFFFFFFFF


def _settings():
    return KernelSettings(flags=tr.TR_FLAG_REFERENCE_SAMPLING | TR_FLAG_REFERENCE_DRAW_RTL)


def _camera(c):
    return CameraSpec(position=tuple(c[0:3]), target=tuple(c[3:6]), up=tuple(c[6:9]), fov=float(c[9]),
                      aperture=float(c[10]), distortion=float(c[11]), focal_dist=float(c[12]),
                      bokeh_side_count=int(c[13]), bokeh_rotation=float(c[14]))


def _case(g, name):
    scene = SCENES[name]()
    assert scene.digest() == str(g[f"{name}_digest"]), "scene generator drifted from the fixture"
    return scene, _camera(g[f"{name}_camera"]), g[f"{name}_pixels"], g[f"{name}_result"]


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", list(SCENES))
def test_oracle_pick_matches_reference_fixture(golden, name):
    scene, cam, px, want = _case(golden, name)
    Oracle.set_reference_draw_order(True)
    try:
        o = Oracle(scene)
        got = np.stack([o.pick_ray(cam, _settings(), scene.width, scene.height, x, y) for x, y in px])
    finally:
        Oracle.set_reference_draw_order(False)
    np.testing.assert_array_equal(got.view(np.uint32), want)
    # the cases cover hits and (heightfield) misses
    assert (want[:, 7] != MISS).any()
    if name == "heightfield_lens":
        assert (want[:, 7] == MISS).any()


@pytest.mark.skipif(not reference_available(), reason="reference host build absent (sources not present)")
def test_reference_pick_reproduces_fixture(golden):
    scene, cam, px, want = _case(golden, "instanced_cornell")
    ref = Reference(scene)
    got = np.stack([ref.pick_ray(cam, _settings(), scene.width, scene.height, x, y) for x, y in px[::7]])
    np.testing.assert_array_equal(got.view(np.uint32), want[::7])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(SCENES))
def test_gpu_pick_matches_reference_fixture(golden, name):
    scene, cam, px, want = _case(golden, name)
    r = tr.DeviceRenderer(0)
    try:
        r.UpdateScene(scene)
        r.SetCamera(cam)
        r.Resize((scene.width, scene.height))
        r.SetSettings(_settings())
        picks = [r.PickRay((int(x), int(y))) for x, y in px]
        stats = r.Statistics()
    finally:
        r.close()
    assert stats["device_error"] == 0
    wf = want.view(np.float32)
    origin = np.array([p.rayOrigin for p in picks], np.float32)
    np.testing.assert_array_equal(origin, wf[:, 0:3])  # the camera position, as the reference reports it
    dirs = np.array([p.rayDir for p in picks], np.float32)
    np.testing.assert_allclose(dirs, wf[:, 4:7], rtol=0, atol=2e-6)
    ids = np.array([(p.instIx, p.primIx) for p in picks], np.uint32)
    same = (ids == want[:, [3, 7]]).all(1)
    # a direction a last bit apart may cross a triangle edge: allow one pick in fifty to land on
    # the neighbouring triangle (at nearly the same distance); misses must agree exactly
    assert same.mean() >= 0.98, same.mean()
    np.testing.assert_array_equal(ids[:, 1] == MISS, want[:, 7] == MISS)
    tmax = np.array([p.tmax for p in picks], np.float32)
    np.testing.assert_allclose(tmax[same], wf[same, 8], rtol=1e-5)
    np.testing.assert_allclose(tmax[~same], wf[~same, 8], rtol=1e-2)
    assert all(p.hit == (p.primIx != MISS) for p in picks)
