"""Batched rendering (tr_batch_*): many scenes of different size, resolution and
sample count in one wavefront, checked against rendering each scene on its own
through tr_render_frame. Random numbers are keyed by (pixel, sample, bounce,
seed) in both and each item keeps its own BVH, so every path takes the same
decisions; the batch kernels are separate template instances whose multiply-adds
the compiler may contract differently, so images agree to a few ulps (2e-6
relative) when the accumulation order is the same."""
import numpy as np
import pytest

import trayracer_gb300 as tr
from trayracer_gb300._abi import TR_FLAG_COUNT_TRAVERSAL
from trayracer_gb300.renderer import KernelSettings

pytestmark = pytest.mark.gpu


def _scenes(res=None):
    out = [
        tr.sphere_scene(5, 3000, 48, 40, 4, 3),
        tr.cornell_box(width=32, height=32, spp=2, max_depth=6),
        tr.sphere_scene(6, 20000, 64, 64, 3, 9),
        tr.sphere_scene(7, 1200, 40, 24, 5, 1),
    ]
    if res is not None:
        for s in out:
            s.width, s.height = res
    return out


def _settings(seed=3):
    return KernelSettings(multiSample=1, maxDepth=6, seed=seed, rrStart=2)


def _single(scene, spp, st, frames=1):
    """Image of one scene through tr_render_frame: `frames` frames of spp / frames samples."""
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene)
    r.SetCamera(scene.camera)
    r.Resize((scene.width, scene.height))
    s = KernelSettings(**{**st.__dict__, "multiSample": spp // frames})
    r.SetSettings(s)
    rays = 0
    for _ in range(frames):
        r.RenderFrame()
        stats = r.Statistics()
        rays += stats["path_count"]
        assert stats["device_error"] == 0
    img = r.ColorBuffer().copy()
    r.close()
    return img, rays


def test_batch_equals_single_scene_renders():
    scenes = _scenes()
    st = _settings()
    with tr.BatchRenderer(scenes) as b:
        info = b.Info()
        assert info["wave_count"] == 1 and info["item_count"] == len(scenes)
        assert info["path_count"] == sum(s.width * s.height * s.spp for s in scenes)
        b.Render(st)
        stats = b.Statistics()
        assert stats["device_error"] == 0
        rays = 0
        for i, s in enumerate(scenes):
            want, n = _single(s, s.spp, st)
            rays += n
            got = b.Image(i)
            np.testing.assert_allclose(got, want, rtol=2e-6, atol=1e-7)
        assert stats["extend_rays"] + stats["shadow_rays"] == rays


def test_batch_split_into_waves_equals_frame_sequence():
    # one sample of one item per wave: the batch adds samples in the order a
    # sequence of one-sample frames does
    scenes = _scenes(res=(32, 24))
    st = _settings(seed=9)
    with tr.BatchRenderer(scenes, wave_paths=32 * 24) as b:
        assert b.Info()["wave_count"] == sum(s.spp for s in scenes)
        b.Render(st, use_graph=True)
        imgs = [b.Image(i).copy() for i in range(len(scenes))]
        b.Render(st, use_graph=False)  # eager replay of the same launches
        for i, s in enumerate(scenes):
            np.testing.assert_array_equal(b.Image(i), imgs[i])
            want, _ = _single(s, s.spp, st, frames=s.spp)
            np.testing.assert_allclose(imgs[i], want, rtol=2e-6, atol=1e-7)


def test_batch_uneven_waves_close_to_single():
    # waves that cut items at arbitrary sample counts: same samples, another summation order
    scenes = _scenes()
    st = _settings(seed=4)
    with tr.BatchRenderer(scenes, wave_paths=5000) as b:
        assert b.Info()["wave_count"] > 2
        b.Render(st)
        for i, s in enumerate(scenes):
            want, _ = _single(s, s.spp, st)
            got = b.Image(i)
            assert np.allclose(got, want, rtol=1e-5, atol=1e-6)


def test_batch_counting_and_errors():
    scenes = _scenes()
    st = _settings()
    with tr.BatchRenderer(scenes) as b:
        cnt = KernelSettings(**{**st.__dict__, "flags": TR_FLAG_COUNT_TRAVERSAL})
        b.Render(cnt)
        s = b.Statistics()
        assert s["traversal_extend_nodes"] > s["extend_rays"] and s["traversal_connect_nodes"] > 0
        bad = KernelSettings(**{**st.__dict__, "flags": tr.TR_FLAG_REFERENCE_SAMPLING})
        with pytest.raises(tr.TracerError):
            b.Render(bad)
        lib = tr.load_library()
        buf = np.empty(16, np.float32)
        assert lib.tr_batch_download(b._b, None, len(scenes), buf.ctypes.data, buf.nbytes) == 1
        assert lib.tr_batch_download(b._b, None, 0, buf.ctypes.data, buf.nbytes) == 1  # buffer too small
    with pytest.raises(tr.TracerError) as e:
        tr.BatchRenderer(scenes, wave_paths=100)  # an item larger than a wave
    assert e.value.status == 6
