"""Textures and normal maps (GetColor / GetIntersectionAttributes, CudaMaterial.h:77-95, 153-191;
Texture::Upload, Texture.cpp:83-139) against frames of the reference's kernels on the textured
Cornell box (tests/golden/ref_textures.npz, tests/golden/make_golden.py textures), whose tex2D
fetches the oracle's restatement of the texture unit's bilinear filter serves: the oracle on the
CPU, the library (the GPU's own texture unit) on the GPU."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle, Reference, reference_available
from trayracer_gb300 import _abi
from trayracer_gb300._abi import TR_FLAG_REFERENCE_DRAW_RTL
from trayracer_gb300.renderer import KernelSettings, RenderModes, SceneDescHolder

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_textures.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _scene(g):
    scene = tr.textured_cornell(width=int(g["width"]), height=int(g["height"]), wall_closure=tr.TR_CLOSURE_LAMBERT)
    assert scene.digest() == str(g["digest"]), "scene generator drifted from the fixture"
    return scene


def _settings(g):
    return KernelSettings(multiSample=1, maxDepth=5, seed=int(g["seed"]), rrStart=1,
                          flags=tr.TR_FLAG_REFERENCE_SAMPLING | TR_FLAG_REFERENCE_DRAW_RTL)


def test_texture_filter_properties():
    """Texel centres return the texel; whole-number shifts of (u, v) wrap to the same value; half
    way between two texels is their mean; the weights take 8 fractional bits."""
    scene = tr.textured_cornell()
    o = Oracle(scene)
    t = scene.textures[1].astype(np.float32)  # 8 x 12
    h, w = t.shape[:2]
    for (i, j) in [(0, 0), (3, 5), (11, 7)]:
        u, v = (i + 0.5) / w, (j + 0.5) / h
        np.testing.assert_array_equal(o.texture_sample(1, u, v), t[j, i])
        np.testing.assert_array_equal(o.texture_sample(1, u + 2.0, v - 3.0), t[j, i])
    mid = o.texture_sample(1, 4.0 / w, 2.5 / h)  # between texels 3 and 4 of row 2
    np.testing.assert_allclose(mid, 0.5 * (t[2, 3] + t[2, 4]), rtol=1e-6)
    # the left edge interpolates with the right-most column (wrap addressing)
    edge = o.texture_sample(1, 0.0, 2.5 / h)
    np.testing.assert_allclose(edge, 0.5 * (t[2, 0] + t[2, w - 1]), rtol=1e-6)
    # a weight of 0.3 is held as 77/256
    q = o.texture_sample(1, (3.5 + 0.3) / w, 2.5 / h)
    np.testing.assert_allclose(q, (1 - 77 / 256) * t[2, 3] + (77 / 256) * t[2, 4], rtol=1e-6)


def test_oracle_matches_reference_fixture(golden):
    scene = _scene(golden)
    Oracle.set_reference_draw_order(True)
    try:
        got, _, _ = Oracle(scene).render(scene.camera, _settings(golden), scene.width, scene.height, frames=1,
                                         threads=1)
    finally:
        Oracle.set_reference_draw_order(False)
    np.testing.assert_array_equal(got[:, :3], golden["frame"][:, :3].astype(np.float64))
    # the textures change the image
    plain = tr.cornell_box(seed=5, width=scene.width, height=scene.height, wall_closure=tr.TR_CLOSURE_LAMBERT)
    Oracle.set_reference_draw_order(True)
    try:
        p, _, _ = Oracle(plain).render(plain.camera, _settings(golden), plain.width, plain.height, frames=1,
                                       threads=1)
    finally:
        Oracle.set_reference_draw_order(False)
    assert not np.allclose(p[:, :3], got[:, :3])


@pytest.mark.skipif(not reference_available(), reason="reference host build absent (sources not present)")
def test_fixture_reproduced_by_reference(golden):
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN.parent / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    try:
        fresh = mg.texture_frames(int(golden["width"]), int(golden["height"]), int(golden["seed"]))
    finally:
        Reference.set_render_mode(7)
    for k in ["frame"] + [f"mode_{m}_{f}" for m, f in golden["modes"]]:
        np.testing.assert_array_equal(fresh[k], golden[k], err_msg=k)


def test_invalid_textures_rejected_by_host_entry():
    lib = _abi.load_library()
    scene = tr.textured_cornell()
    O = np.zeros((1, 4), np.float32)
    hits = np.zeros((1, 4), np.uint32)

    def status(mutate):
        sc = tr.textured_cornell()
        mutate(sc)
        h = SceneDescHolder(sc)
        return lib.tr_trace_host(C.byref(h.desc), O.ctypes.data, O.ctypes.data, 1, 1e-3, 0, hits.ctypes.data, None)

    assert status(lambda sc: None) == 0
    assert status(lambda sc: sc.material_textures.__setitem__((0, 3), 9)) == 1        # missing texture
    assert status(lambda sc: sc.material_textures.__setitem__((0, 4), 0)) == 1        # emissive takes none
    assert status(lambda sc: sc.textures.__setitem__(0, np.zeros((0, 4, 4), np.float16))) == 1  # empty
    assert scene.material_textures.shape == (scene.materials.shape[0], 13)


def _gpu(scene, st, mode=RenderModes.PathTracing, flags=0):
    r = tr.DeviceRenderer(0)
    try:
        r.UpdateScene(scene)
        r.SetCamera(scene.camera)
        r.Resize((scene.width, scene.height))
        r.RenderFrame(st, mode, flags)
        acc = r.Accumulator().reshape(-1, 4).copy()
        stats = r.Statistics()
    finally:
        r.close()
    assert stats["device_error"] == 0
    return acc


@pytest.mark.gpu
@pytest.mark.parametrize("mode,flags", [(5, 3), (5, 5), (5, 6), (5, 7), (8, 0)])
def test_gpu_texture_fetches_match_reference(golden, mode, flags):
    """The texture unit against the restated filter: a property image is the stored colour times
    the filtered texel, so the two agree to the weights' 8-bit steps."""
    scene = _scene(golden)
    acc = _gpu(scene, _settings(golden), RenderModes(mode), flags)
    want = golden[f"mode_{mode}_{flags}"]
    diff = np.abs(acc[:, :3] - want[:, :3])
    print(f"mode {mode}/{flags}: max |gpu - oracle filter| = {diff.max():.3e}")
    ok = (diff <= 4e-3 + 1e-3 * np.abs(want[:, :3])).all(1)
    assert ok.mean() >= 0.99, ok.mean()
    np.testing.assert_array_equal(acc[:, 3], want[:, 3])


@pytest.mark.gpu
def test_gpu_textured_frame_matches_reference(golden):
    scene = _scene(golden)
    acc = _gpu(scene, _settings(golden))
    want = golden["frame"]
    ok = np.isclose(acc[:, :3], want[:, :3], rtol=1e-2, atol=1e-4).all(1)
    assert ok.mean() >= 0.97, ok.mean()
    assert abs(acc[:, :3].mean() - want[:, :3].mean()) <= 1e-2 * want[:, :3].mean()


@pytest.mark.gpu
def test_gpu_textured_default_sampling_per_path():
    scene = tr.textured_cornell(width=40, height=30)
    st = tr.settings_for(scene, multi_sample=2)
    r = tr.DeviceRenderer(0)
    try:
        r.UpdateScene(scene)
        r.SetCamera(scene.camera)
        r.Resize((scene.width, scene.height))
        r.RenderFrame(st)
        buf = r.Buffers()
        rad = r.read_device(buf["radiance"], np.float32, buf["capacity"] * 4).reshape(2, -1, 4)
        # updating the materials keeps the textures
        r.UpdateMaterials(scene.materials)
        r.RenderFrame(st)
        stats = r.Statistics()
    finally:
        r.close()
    assert stats["device_error"] == 0
    _, paths, _ = Oracle(scene).render(scene.camera, st, scene.width, scene.height, want_paths=True)
    ok = np.isclose(rad[..., :3].astype(np.float64), paths[..., :3], rtol=1e-2, atol=1e-4).all(-1)
    assert ok.mean() >= 0.97, ok.mean()
