"""The Preetham sky seen by paths that leave the scene (SampleSky, CudaSky.h:105-156, called from
PathTracing.h:40-55) against frames of the reference's own kernels (tests/golden/ref_sky.npz, made
by tests/golden/make_golden.py sky): the oracle on the CPU, the library on the GPU."""
from pathlib import Path

import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle, Reference, reference_available
from trayracer_gb300._abi import TR_FLAG_REFERENCE_DRAW_RTL
from trayracer_gb300.renderer import KernelSettings

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_sky.npz"
SKY_CASES = {
    "sun_high": dict(sunDir=(0.2, 0.9, 0.4)),
    "sun_low": dict(sunDir=(0.4, 0.15, 0.8), turbidity=6.5, sunAngularDiameter=300.0),
    "sun_set": dict(sunDir=(0.0, -0.2, 1.0), drawSun=False),
}


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _scene(g):
    scene = tr.outdoor_heightfield(width=int(g["width"]), height=int(g["height"]), lambert=True)
    assert scene.digest() == str(g["digest"]), "scene generator drifted from the fixture"
    return scene


def _ref_settings(g, ms=1):
    return KernelSettings(multiSample=ms, maxDepth=int(g["max_depth"]), seed=int(g["seed"]), rrStart=1,
                          flags=tr.TR_FLAG_REFERENCE_SAMPLING | TR_FLAG_REFERENCE_DRAW_RTL)


@pytest.mark.parametrize("case", list(SKY_CASES))
def test_oracle_sky_matches_reference_fixture(golden, case):
    """Bit for bit at one sample per pixel (same operations, same order; host libm)."""
    scene = _scene(golden)
    Oracle.set_reference_draw_order(True)
    try:
        o = Oracle(scene)
        o.set_sky(tr.SkySettings(**SKY_CASES[case]))
        got, _, _ = o.render(scene.camera, _ref_settings(golden), scene.width, scene.height, frames=1, threads=1)
        o.set_sky(None)
        dark, _, _ = o.render(scene.camera, _ref_settings(golden), scene.width, scene.height, frames=1, threads=1)
    finally:
        Oracle.set_reference_draw_order(False)
    want = golden[f"{case}_acc"]
    np.testing.assert_array_equal(got[:, :3], want[:, :3].astype(np.float64))
    # the sky lights the scene: the frame is brighter than without it
    assert want[:, :3].mean() > dark[:, :3].mean()


@pytest.mark.skipif(not reference_available(), reason="reference host build absent (sources not present)")
def test_oracle_sky_matches_reference_live_two_samples(golden):
    scene = _scene(golden)
    sky = tr.SkySettings(sunDir=(-0.3, 0.4, 0.5), turbidity=2.0, sunIntensity=400.0)
    st = _ref_settings(golden, ms=2)
    ref = Reference(scene)
    ref.set_sky(sky)
    acc = np.zeros((scene.width * scene.height, 4), np.float32)
    ref.render_frame(scene.camera, st, scene.width, scene.height, 0, acc)
    Oracle.set_reference_draw_order(True)
    try:
        o = Oracle(scene)
        o.set_sky(sky)
        got, _, _ = o.render(scene.camera, st, scene.width, scene.height, frames=1, threads=1)
    finally:
        Oracle.set_reference_draw_order(False)
    # two samples: the reference adds them into float32 pixels, the oracle in double
    np.testing.assert_allclose(got[:, :3], acc[:, :3].astype(np.float64), rtol=2e-6, atol=1e-7)


def _gpu_frame(scene, st, sky, use_graph=False, aovs=False):
    r = tr.DeviceRenderer(0)
    try:
        r.UpdateScene(scene)
        r.SetCamera(scene.camera)
        r.Resize((scene.width, scene.height))
        r.SetSky(sky)
        if aovs:
            st = KernelSettings(**{**st.__dict__, "flags": st.flags | tr.TR_FLAG_WRITE_AOVS})
        r.RenderFrame(st, use_graph=use_graph)
        acc = r.Accumulator().reshape(-1, 4).copy()
        buf = r.Buffers()
        rad = r.read_device(buf["radiance"], np.float32, buf["capacity"] * 4).reshape(-1, 4).copy()
        albedo = r.read_device(buf["albedo"], np.float32, scene.width * scene.height * 4).reshape(-1, 4).copy()
        stats = r.Statistics()
    finally:
        r.close()
    assert stats["device_error"] == 0
    return acc, rad, albedo


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(SKY_CASES))
@pytest.mark.parametrize("use_graph", [False, True])
def test_gpu_sky_matches_reference_fixture(golden, case, use_graph):
    """Reference sampling: the same paths as the reference's kernels; the sky terms round
    differently (device powf/expf/acosf against the host's), so per pixel within 1e-4."""
    scene = _scene(golden)
    acc, _, _ = _gpu_frame(scene, _ref_settings(golden), tr.SkySettings(**SKY_CASES[case]), use_graph)
    want = golden[f"{case}_acc"]
    ok = np.isclose(acc[:, :3], want[:, :3], rtol=1e-4, atol=1e-6).all(1)
    # a last-bit difference in a hit distance can send a path elsewhere
    assert ok.mean() >= 0.99, ok.mean()
    assert abs(acc[:, :3].mean() - want[:, :3].mean()) <= 2e-3 * want[:, :3].mean()
    np.testing.assert_array_equal(acc[:, 3], want[:, 3])


@pytest.mark.gpu
def test_gpu_sky_default_sampling_per_path():
    """Default sampling (counter RNG, MIS): every path's radiance against the oracle's."""
    scene = tr.outdoor_heightfield(width=40, height=30)
    sky = tr.SkySettings(sunDir=(0.4, 0.3, 0.8), turbidity=3.0)
    st = tr.settings_for(scene, multi_sample=2)
    st = KernelSettings(**{**st.__dict__, "maxDepth": 4})
    _, rad, _ = _gpu_frame(scene, st, sky)
    o = Oracle(scene)
    o.set_sky(sky)
    _, paths, _ = o.render(scene.camera, st, scene.width, scene.height, want_paths=True)
    got = rad[:, :3].astype(np.float64).reshape(paths[..., :3].shape)
    ok = np.isclose(got, paths[..., :3], rtol=1e-3, atol=1e-5).all(-1)
    assert ok.mean() >= 0.98, ok.mean()
    assert paths[..., :3].mean() > 0


@pytest.mark.gpu
def test_gpu_sky_albedo_guide_and_disable():
    """A primary miss writes the sky as its albedo guide; tr_set_sky(NULL) makes misses black again."""
    scene = tr.outdoor_heightfield(width=32, height=24)
    st = tr.settings_for(scene, multi_sample=1)
    sky = tr.SkySettings(sunDir=(0.0, 0.5, 1.0))
    acc_sky, _, albedo = _gpu_frame(scene, st, sky, aovs=True)
    acc_dark, _, albedo_dark = _gpu_frame(scene, st, None, aovs=True)
    assert acc_sky[:, :3].mean() > acc_dark[:, :3].mean()
    # the top rows look above the horizon: their guide albedo is the (non-zero) sky there
    top = albedo.reshape(scene.height, scene.width, 4)[-1, :, :3]
    assert (top > 0).all()
    assert (albedo_dark.reshape(scene.height, scene.width, 4)[-1, :, :3] == 0).all()


@pytest.mark.gpu
def test_gpu_sky_arguments_and_adjoint():
    scene = tr.outdoor_heightfield(width=16, height=12)
    r = tr.DeviceRenderer(0)
    try:
        r.UpdateScene(scene)
        r.SetCamera(scene.camera)
        r.Resize((scene.width, scene.height))
        with pytest.raises(tr.TracerError):
            r.SetSky(tr.SkySettings(sunDir=(0.0, 0.0, 0.0)))
        with pytest.raises(tr.TracerError):
            r.SetSky(tr.SkySettings(sunIntensity=float("nan")))
        r.SetSky(tr.SkySettings())
        r.RenderFrame(tr.settings_for(scene, multi_sample=1))
        # the path-replay adjoint differentiates scenes without a sky (refused before any launch;
        # the buffers are real so that nothing could read out of bounds if it were not)
        torch = pytest.importorskip("torch")
        pg = torch.ones((scene.height, scene.width, 4), dtype=torch.float32, device="cuda")
        grad = torch.zeros((scene.materials.shape[0], 9), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        with pytest.raises(tr.TracerError):
            r.AdjointFrame(pg.data_ptr(), 1.0, grad.data_ptr())
        assert float(grad.abs().sum()) == 0.0
    finally:
        r.close()
