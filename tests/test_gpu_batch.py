"""Batched rendering (tr_batch_*): many scenes of different size, resolution and
sample count in one continuous wavefront (a pool of path slots refilled with new
samples as paths end), checked against rendering each scene on its own through
tr_render_frame with multi_sample = spp. Random numbers are keyed by (pixel,
sample, bounce, seed) in both, each item keeps its own BVH and each pixel's
samples are summed in sample order, so every path takes the same decisions and
the images agree to a few ulps (2e-6 relative: the batch kernels are separate
template instances whose multiply-adds the compiler may contract differently),
whatever the pool size."""
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


@pytest.mark.parametrize("pool", [0, 5000, 700])
def test_batch_equals_single_scene_renders(pool):
    """Default pool (larger than the batch: one iteration per bounce), and pools smaller than
    one item's pixels (many iterations, paths of different bounces in one queue)."""
    scenes = _scenes()
    st = _settings()
    with tr.BatchRenderer(scenes, pool_paths=pool) as b:
        info = b.Info()
        total = sum(s.width * s.height * s.spp for s in scenes)
        assert info["round_count"] == 1 and info["item_count"] == len(scenes)
        assert info["path_count"] == total
        assert info["pool_paths"] == (min(pool, total) if pool else total)
        b.Render(st)
        stats = b.Statistics()
        assert stats["device_error"] == 0
        if pool:
            assert stats["iterations"] > total // pool
        rays = 0
        for i, s in enumerate(scenes):
            want, n = _single(s, s.spp, st)
            rays += n
            got = b.Image(i)
            np.testing.assert_allclose(got, want, rtol=2e-6, atol=1e-7)
        assert stats["extend_rays"] + stats["shadow_rays"] == rays
        assert stats["launches"] == 1 + 4 * (stats["iterations"] + 1)


def test_batch_graph_equals_eager():
    # the graph's device-driven while loop and the host-driven iterations run the same launches
    scenes = _scenes(res=(32, 24))
    st = _settings(seed=9)
    with tr.BatchRenderer(scenes, pool_paths=1000) as b:
        b.Render(st, use_graph=True)
        imgs = [b.Image(i).copy() for i in range(len(scenes))]
        g = b.Statistics()
        b.Render(st, use_graph=False)
        e = b.Statistics()
        for i in range(len(scenes)):
            np.testing.assert_array_equal(b.Image(i), imgs[i])
        assert (g["iterations"], g["extend_rays"], g["shadow_rays"]) == (e["iterations"], e["extend_rays"],
                                                                          e["shadow_rays"])
        b.Render(st, use_graph=True)  # replay
        for i in range(len(scenes)):
            np.testing.assert_array_equal(b.Image(i), imgs[i])


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
        tr.BatchRenderer(scenes, pool_paths=1 << 28)  # more path slots than path indices
    assert e.value.status == 6


def test_batch_with_textured_items():
    """Textured items (textures and normal maps) batch beside untextured ones; each image
    equals the item's single-scene render (a last-bit difference in a hit point moves a
    bilinear lookup: measured 2 pixels of 1200 beyond 2e-6, one dim channel 4.2e-6 off in
    absolute terms; 99.5 % of pixels within 1e-5 relative and all within 1e-3 relative or
    1e-5 absolute)."""
    scenes = [tr.textured_cornell(width=40, height=30, spp=4), tr.sphere_scene(5, 3000, 48, 40, 4, 3),
              tr.textured_cornell(seed=9, width=24, height=24, spp=2)]
    st = _settings()
    with tr.BatchRenderer(scenes) as b:
        b.Render(st)
        assert b.Statistics()["device_error"] == 0
        for i, s in enumerate(scenes):
            want, _ = _single(s, s.spp, st)
            got = b.Image(i)
            close = np.isclose(got, want, rtol=1e-5, atol=1e-7).all(-1)
            assert close.mean() >= 0.995, (i, close.mean())
            np.testing.assert_allclose(got, want, rtol=1e-3, atol=1e-5)
