"""The CPU oracle pinned to the reference: golden fixtures made by the
reference's own code (tests/golden, make_golden.py) and, where the reference
sources are present, the reference's kernels compiled as host C++."""
from pathlib import Path

import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle, Reference, reference_available
from trayracer_gb300._abi import TR_FLAG_REFERENCE_DRAW_RTL
from trayracer_gb300.renderer import KernelSettings

GOLDEN = Path(__file__).resolve().parent / "golden"


def _ref_settings(ms, seed, rtl=True):
    flags = tr.TR_FLAG_REFERENCE_SAMPLING | (TR_FLAG_REFERENCE_DRAW_RTL if rtl else 0)
    return KernelSettings(multiSample=ms, maxDepth=5, seed=seed, rrStart=1, flags=flags)


@pytest.fixture(autouse=True)
def _draw_order():
    Oracle.set_reference_draw_order(False)
    yield
    Oracle.set_reference_draw_order(False)


def test_reference_rng_golden():
    g = np.load(GOLDEN / "ref_rng.npz")
    for (a, b), draws in zip(g["pairs"], g["draws"]):
        np.testing.assert_array_equal(Oracle.reference_rng(int(a), int(b), draws.size), draws)


@pytest.mark.parametrize("name,ctype", [("lambert", tr.TR_CLOSURE_LAMBERT), ("diffuse", tr.TR_CLOSURE_DIFFUSE),
                                        ("disney", tr.TR_CLOSURE_DISNEY)])
def test_closures_golden(name, ctype):
    g = np.load(GOLDEN / "ref_closures.npz")
    x, want = g[f"{name}_in"], g[f"{name}_out"]
    got = Oracle.closure(ctype, x, reference=True)
    # flags are bit patterns, compare exactly; values to 1e-6 relative (the oracle
    # and the reference build round at the same places, so most are identical)
    np.testing.assert_array_equal(got[:, 7].view(np.uint32), want[:, 7].view(np.uint32))
    vals = np.delete(np.arange(14), [7, 12, 13])
    np.testing.assert_allclose(got[:, vals], want[:, vals], rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("fixture", ["ref_cornell_32x32_ms1.npz", "ref_cornell_24x16_ms2.npz"])
def test_frames_golden(fixture):
    """The oracle's frame loop reproduces the reference's accumulator bit for bit
    (reference sampling, right-to-left argument draws as the host build takes them)."""
    g = np.load(GOLDEN / fixture)
    w, h, ms, seed = int(g["width"]), int(g["height"]), int(g["ms"]), int(g["seed"])
    scene = tr.cornell_box(wall_closure=tr.TR_CLOSURE_LAMBERT, width=w, height=h)
    assert scene.digest() == str(g["digest"]), "scene generator drifted from the fixture"
    Oracle.set_reference_draw_order(True)
    o = Oracle(scene)
    st = _ref_settings(ms, seed)
    # first frame: with one sample per pixel both sum a path's contributions
    # into one float in the same order, so the result is identical
    acc1, _, _ = o.render(scene.camera, st, w, h, frames=1, threads=1)
    want1 = g["acc"][0].astype(np.float64)
    tol = 0 if ms == 1 else 2e-6
    np.testing.assert_allclose(acc1[:, :3], want1[:, :3], rtol=tol, atol=tol)
    # all frames: the reference accumulates into float32 pixels, the oracle in double
    acc, _, _ = o.render(scene.camera, st, w, h, frames=int(g["frames"]), threads=1)
    want = g["acc"][-1].astype(np.float64)
    np.testing.assert_allclose(acc[:, :3], want[:, :3], rtol=2e-6, atol=1e-6)
    np.testing.assert_array_equal(acc[:, 3], want[:, 3])


def test_stage_golden_primary_and_shade():
    g = np.load(GOLDEN / "ref_cornell_32x32_ms1.npz")
    w, h, seed = int(g["width"]), int(g["height"]), int(g["seed"])
    scene = tr.cornell_box(wall_closure=tr.TR_CLOSURE_LAMBERT, width=w, height=h)
    Oracle.set_reference_draw_order(True)
    o = Oracle(scene)
    st = _ref_settings(1, seed)
    O, D, T = o.generate(scene.camera, st, w, h, 0, 0, w * h)
    ps = g["prim_states"]
    np.testing.assert_array_equal(O, ps[0])
    np.testing.assert_array_equal(D, ps[1])
    np.testing.assert_array_equal(T, ps[2])
    hits = o.trace_closest(ps[0], ps[1], st.rayEpsilon)
    np.testing.assert_array_equal(hits, g["prim_hits"])
    ext, ev, sh, sv, rad = o.shade(st, 0, 0, w, h, ps[0], ps[1], ps[2], g["prim_hits"])
    # the reference compacts extend and shadow rays in job order (sequential host run)
    got_ext = ext[ev].transpose(1, 0, 2)
    want_ext = g["shade_states"]
    np.testing.assert_array_equal(got_ext[0], want_ext[0])
    np.testing.assert_array_equal(got_ext[2], want_ext[2])
    # D.w carries PackNormal (CudaUtility.h:153-160), which nothing reads; its
    # float->uint conversion of negative components is undefined in C++ (the host
    # build wraps, the GPU saturates), so only the direction is compared
    np.testing.assert_array_equal(got_ext[1][:, :3], want_ext[1][:, :3])
    got_sh = sh[sv].transpose(1, 0, 2)
    np.testing.assert_array_equal(got_sh[:2], g["shade_shadow"][:2])
    np.testing.assert_array_equal(got_sh[2, :, :3], g["shade_shadow"][2, :, :3])


@pytest.mark.skipif(not reference_available(), reason="reference host build absent (sources not present)")
def test_oracle_matches_reference_kernels_live():
    """Against the live reference build on a fresh seed and resolution (both modes of draw order)."""
    scene = tr.cornell_box(wall_closure=tr.TR_CLOSURE_LAMBERT, width=20, height=12)
    Oracle.set_reference_draw_order(True)
    st = _ref_settings(1, 4242)
    ref = Reference(scene)
    acc = np.zeros((20 * 12, 4), np.float32)
    ref.render_frame(scene.camera, st, 20, 12, 0, acc)
    o = Oracle(scene)
    got, _, _ = o.render(scene.camera, st, 20, 12, frames=1, threads=1)
    np.testing.assert_array_equal(got[:, :3], acc[:, :3].astype(np.float64))
    for f in range(1, 3):
        ref.render_frame(scene.camera, st, 20, 12, f, acc)
    got, _, _ = o.render(scene.camera, st, 20, 12, frames=3, threads=1)
    np.testing.assert_allclose(got[:, :3], acc[:, :3].astype(np.float64), rtol=2e-6, atol=1e-6)


@pytest.mark.skipif(not reference_available(), reason="reference host build absent (sources not present)")
def test_oracle_matches_reference_kernels_two_level():
    """Two-level scene (meshes placed by instances): the reference's kernels read the mesh of
    the hit instance, its material offset and its inverse transform (CudaMaterial.h:123-211)."""
    scene = tr.instanced_cornell(wall_closure=tr.TR_CLOSURE_LAMBERT, width=24, height=16)
    Oracle.set_reference_draw_order(True)
    ref = Reference(scene)
    o = Oracle(scene)
    for ms, tol in ((1, 0.0), (2, 2e-6)):
        # one sample per pixel: both sum a path's contributions in the same order; two: the
        # reference adds the samples into float32 pixels, the oracle in double
        st = _ref_settings(ms, 91)
        acc = np.zeros((24 * 16, 4), np.float32)
        ref.render_frame(scene.camera, st, 24, 16, 0, acc)
        got, _, _ = o.render(scene.camera, st, 24, 16, frames=1, threads=1)
        np.testing.assert_allclose(got[:, :3], acc[:, :3].astype(np.float64), rtol=tol, atol=tol)
        assert acc[:, :3].max() > 0


@pytest.mark.skipif(not reference_available(), reason="reference host build absent (sources not present)")
def test_debug_mode_fixture_reproduced_by_reference():
    """ref_debug_modes.npz is what the reference's other shade kernels make today."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = np.load(GOLDEN / "ref_debug_modes.npz")
    try:
        fresh = mg.debug_mode_frames(int(g["width"]), int(g["height"]), int(g["seed"]), float(g["ao_dist"]),
                                     float(g["z_depth_max"]))
    finally:
        Reference.set_render_mode(7)
    for mode, flags in g["modes"]:
        key = f"mode_{mode}_{flags}"
        np.testing.assert_array_equal(fresh[key], g[key], err_msg=key)
    # the modes are not all alike: normals, IDs and depth differ from one another
    assert len({g[f"mode_{m}_{f}"].tobytes() for m, f in g["modes"]}) >= 12


def test_counter_rng_properties():
    u = np.concatenate([Oracle.counter_rng(p, s, b, 1, 8) for p in range(64) for s in range(4) for b in range(3)])
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.02
    # 24-bit values
    assert np.all((u * 16777216.0) == np.floor(u * 16777216.0))
    # different keys, different streams; same key, same stream
    np.testing.assert_array_equal(Oracle.counter_rng(3, 4, 5, 6, 10), Oracle.counter_rng(3, 4, 5, 6, 10))
    assert not np.array_equal(Oracle.counter_rng(3, 4, 5, 6, 10), Oracle.counter_rng(3, 4, 6, 6, 10))
    assert not np.array_equal(Oracle.counter_rng(3, 4, 5, 6, 10), Oracle.counter_rng(3, 5, 5, 6, 10))
    # decorrelated neighbouring pixels
    a = np.array([Oracle.counter_rng(p, 0, 1, 1, 1)[0] for p in range(4096)])
    assert abs(np.corrcoef(a[:-1], a[1:])[0, 1]) < 0.05


def test_fp64_oracle_close_to_fp32():
    scene = tr.cornell_box(width=24, height=24)
    st = tr.settings_for(scene, multi_sample=4)
    o = Oracle(scene)
    a32, _, _ = o.render(scene.camera, st, 24, 24)
    a64, _, _ = o.render(scene.camera, st, 24, 24, use_double=True)
    i32 = a32[:, :3] / a32[:, 3:4]
    i64 = a64[:, :3] / a64[:, 3:4]
    rmse = np.sqrt(np.mean((i32 - i64) ** 2)) / max(1e-9, np.sqrt(np.mean(i64 ** 2)))
    assert rmse < 5e-2, rmse


def test_alias_table_matches_energy():
    scene = tr.heightfield(n=32, width=16, height=16)
    o = Oracle(scene)
    assert o.light_count == 64
    assert o.light_energy(True) > o.light_energy(False) > 0
