"""tr_render_samples: spp samples per pixel as one continuous wavefront (the
frame's path slots refilled with the next samples as paths end), checked
against the same samples rendered frame by frame with tr_render_frame.

The sample keys are the frames' (pixel, sample, bounce, seed), so every path
takes the same decisions; the continuous kernels are separate template
instances (camera rays made inside extend from the item's camera) whose
multiply-adds the compiler may contract differently, so a path's radiance may
differ in its last bits (measured: 3.5e-6 relative on one pixel of 9216), and
a pixel's spp samples are summed in one run rather than frame by frame:
images agree to 1e-5 relative."""
import dataclasses

import numpy as np
import pytest

import trayracer_gb300 as tr
from trayracer_gb300.renderer import TracerError

pytestmark = pytest.mark.gpu


def renderer(scene, st):
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene)
    r.SetCamera(scene.camera)
    r.Resize((scene.width, scene.height))
    r.SetSettings(st)
    return r


def frames(scene, st, n, sky=None):
    r = renderer(scene, st)
    if sky is not None:
        r.SetSky(sky)
    rays = 0
    for _ in range(n):
        r.RenderFrame(use_graph=True)
        rays += r.Statistics()["path_count"]
    img, acc = r.ColorBuffer().copy(), r.Accumulator().copy()
    r.close()
    return img, acc, rays


SCENES = {
    "heightfield": lambda: tr.heightfield(n=128, width=64, height=36, rr_start=2),
    "cornell": lambda: tr.cornell_box(width=48, height=40),
}


@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("n_frames", [1, 4])
def test_samples_equal_frames(name, n_frames):
    scene = SCENES[name]()
    st = tr.settings_for(scene, multi_sample=4)
    want, want_acc, want_rays = frames(scene, st, n_frames)
    r = renderer(scene, st)
    r.RenderSamples(4 * n_frames)
    got, acc = r.ColorBuffer(), r.Accumulator()
    s = r.Statistics()
    r.close()
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-7)
    np.testing.assert_array_equal(acc[..., 3], want_acc[..., 3])
    assert s["sample_count"] == 4 * n_frames and s["device_error"] == 0
    assert s["primary_path_count"] == scene.width * scene.height * 4 * n_frames
    assert abs(s["path_count"] - want_rays) <= 1e-3 * want_rays


def test_samples_continue_an_accumulation_graph_and_eager():
    scene = SCENES["heightfield"]()
    st = tr.settings_for(scene, multi_sample=2)
    want, _, _ = frames(scene, st, 3)
    r = renderer(scene, st)
    r.RenderFrame()
    r.RenderSamples(4, use_graph=True)
    a = r.ColorBuffer().copy()
    assert r.SampleCount() == 6
    r.Reset()
    r.RenderFrame()
    r.RenderSamples(4, use_graph=False)
    b = r.ColorBuffer().copy()
    r.Reset()
    r.RenderFrame()
    r.RenderSamples(4, use_graph=True)  # graph replay
    c = r.ColorBuffer().copy()
    r.close()
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)
    np.testing.assert_allclose(a, want, rtol=1e-5, atol=1e-7)


def test_samples_with_sky():
    scene = tr.outdoor_heightfield(n=32, width=48, height=32)
    sky = tr.SkySettings(enabled=True, drawSun=True)
    st = tr.settings_for(scene, multi_sample=2)
    want, _, _ = frames(scene, st, 2, sky=sky)
    r = renderer(scene, st)
    r.SetSky(sky)
    r.RenderSamples(4)
    got = r.ColorBuffer()
    r.close()
    assert got[..., :3].mean() > 0
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-7)


def test_samples_textured_scene():
    """Textures and normal maps go through the continuous kernels too (the shade kernel's
    texture variant): the same image as the frames. A last-bit difference in a hit point
    moves a bilinear texture lookup, so a pixel may differ more than elsewhere (measured:
    one pixel of 1600 at 8e-5 relative): 99.9 % of pixels within 1e-5, all within 1e-3."""
    scene = tr.textured_cornell(width=40, height=30)
    st = tr.settings_for(scene, multi_sample=2)
    want, _, want_rays = frames(scene, st, 3)
    r = renderer(scene, st)
    r.RenderSamples(6)
    got = r.ColorBuffer()
    s = r.Statistics()
    r.close()
    assert s["iterations"] > 0  # the continuous wavefront, not the frames
    close = np.isclose(got, want, rtol=1e-5, atol=1e-7).all(-1)
    assert close.mean() >= 0.999, close.mean()
    np.testing.assert_allclose(got, want, rtol=1e-3, atol=1e-6)
    assert abs(s["path_count"] - want_rays) <= 1e-3 * want_rays


def test_samples_two_level_scene():
    """Instanced scenes (two-level traversal) go through the continuous kernels too."""
    scene = tr.instanced_cornell(width=40, height=32)
    st = tr.settings_for(scene, multi_sample=2)
    want, _, want_rays = frames(scene, st, 2)
    r = renderer(scene, st)
    r.RenderSamples(4)
    got = r.ColorBuffer()
    s = r.Statistics()
    r.close()
    assert s["iterations"] > 0 and s["device_error"] == 0
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-7)
    assert abs(s["path_count"] - want_rays) <= 1e-3 * want_rays


def test_samples_fall_back_to_frames():
    # the reference's sampling renders the frames themselves
    scene = tr.cornell_box(width=40, height=32)
    st = tr.settings_for(scene, multi_sample=2, reference=True)
    want, _, _ = frames(scene, st, 2)
    r = renderer(scene, st)
    r.RenderSamples(4)
    got = r.ColorBuffer()
    assert r.Statistics()["iterations"] == 0
    r.close()
    np.testing.assert_array_equal(got, want)


def test_samples_errors():
    scene = SCENES["cornell"]()
    r = renderer(scene, tr.settings_for(scene, multi_sample=4))
    with pytest.raises(TracerError) as e:
        r.RenderSamples(6)  # not a multiple of multi_sample
    assert e.value.status == 1
    r.SetSettings(dataclasses.replace(tr.settings_for(scene, multi_sample=4), traversalStepLimit=2))
    r.RenderSamples(8)
    assert r.Statistics()["device_error"] != 0
    r.close()


def test_samples_statistics():
    """Totals of a continuous render against the same samples as frames, the stage times of an
    eager render (zero after a graph render), and the launch count."""
    scene = SCENES["heightfield"]()
    st = tr.settings_for(scene, multi_sample=2)
    r = renderer(scene, st)
    hits = ext = shadow = 0
    for _ in range(3):
        r.RenderFrame(use_graph=False)
        f = r.Statistics()
        assert f["hit_ray_count"] == sum(f["hit_rays"])
        hits += f["hit_ray_count"]
        ext += f["primary_path_count"] + f["secondary_path_count"] + f["deep_path_count"]
        shadow += f["shadow_ray_count"]
    for graph in (False, True):
        r.Reset()
        r.RenderSamples(6, use_graph=graph)
        s = r.Statistics()
        assert s["device_error"] == 0 and s["iterations"] >= 3  # the pool holds a third of the samples
        assert s["launches"] == 2 + 4 * (s["iterations"] + 1)
        n = s["primary_path_count"] + s["secondary_path_count"]
        assert s["primary_path_count"] == scene.width * scene.height * 6
        assert s["path_count"] == n + s["shadow_ray_count"]
        for got, want in ((n, ext), (s["shadow_ray_count"], shadow), (s["hit_ray_count"], hits)):
            assert abs(got - want) <= 1e-3 * want
        times = [s[f"{k}_time_ms"] for k in ("generate", "extend", "shade", "connect", "finalize")]
        if graph:
            assert all(t == 0 for t in times)
        else:
            assert all(t > 0 for t in times)
            assert s["render_time_ms"] == pytest.approx(sum(times), rel=1e-5)
    r.close()


def test_autotune_on_continuous_renders():
    """tr_autotune with TR_TUNE_SAMPLES times continuous renders; the chosen tuning is applied,
    the accumulation reset, and the continuous render afterwards matches the frames it replaces."""
    scene = tr.cornell_box(width=64, height=48)
    st = tr.settings_for(scene, multi_sample=2)
    r = renderer(scene, st)
    rep = r.Autotune(skip_bvh=True, samples=True)
    assert rep["trials"] >= 10
    assert rep["frame_ms_tuned"] <= rep["frame_ms_default"]
    assert rep["chosen"] == r.Tuning() and r.SampleCount() == 0
    r.RenderSamples(4)
    got = r.ColorBuffer().copy()
    r.close()
    want, _, _ = frames(scene, st, 2)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-7)
