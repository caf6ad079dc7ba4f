"""GPU parity on the benchmarked configurations at their full sizes, through the
C ABI, path by path against the CPU oracle.

plain, large: the 1024 x 1024 value-noise heightfield (2,093,122 triangles with
the 64 emissive ones), 256 Disney materials, 1920 x 1080, 64 samples per pixel
rendered as 4 frames of 16, 8 bounces, Russian roulette from bounce 3 - at the
leaf size the autotuner picks on this scene (3) and at one triangle per leaf.
The oracle renders three windows of 64 x 8 pixels: the image centre, the rows
where the terrain meets the (black) sky, and the near edge of the terrain.

plain, small: the closed box at 256 x 256, 16 samples per pixel, 5 bounces, no
Russian roulette: every path of the frame.

Tolerances are those of the stage-wise parity tests:
  hits       bit-exact primitive, t and 16-bit barycentrics, except logged near
             ties (|dt| <= 1e-6 t) between triangles that share an edge;
  radiance   per path within 1e-4 relative (atol 1e-6) on >= 99.5 % of the
             paths; the rest are paths whose discrete decisions (Russian
             roulette, NEE gate, lobe choice) flipped on a last-bit difference
             of the fp32 arithmetic, which the oracle's own fp32 and fp64 runs
             show as well;
  image      the GPU's relative RMSE against the FP64 oracle is at most
             1.5 x that of the fp32 oracle (+1e-5): the residual is fp32 against
             fp64 path divergence, not a GPU error.
"""
import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle

pytestmark = pytest.mark.gpu

RTOL = 1e-4
N_COUNTERS = 5 * 17
HIT_BASE = 4 * 17
WIN_W, WIN_H = 64, 8
# (x0, y0) of each window; row 0 is the bottom of the image. The horizon and near-edge windows are
# where about half of the camera rays hit the terrain and the rest leave it.
WINDOWS = {"centre": (928, 536), "horizon": (1248, 924), "near_edge": (288, 12)}


def close(a, b, rtol=RTOL, atol=1e-6):
    return np.abs(a - b) <= rtol * np.maximum(1.0, np.abs(b)) + atol


def rel_rmse(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(1e-12, np.sqrt(np.mean(b ** 2))))


@pytest.fixture(scope="module")
def heightfield():
    scene = tr.heightfield()
    assert scene.triangle_count == 1023 * 1023 * 2 + 64
    assert (scene.width, scene.height, scene.spp, scene.max_depth, scene.rr_start) == (1920, 1080, 64, 8, 3)
    return scene, Oracle(scene)


def window_pixels(W):
    """Pixel indices of the windows, row by row: {name: [(first_pixel, count), ...]}."""
    return {k: [((y0 + j) * W + x0, WIN_W) for j in range(WIN_H)] for k, (x0, y0) in WINDOWS.items()}


def renderer(scene, st, leaf_size=0):
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene, leaf_size=leaf_size)
    r.SetCamera(scene.camera)
    r.Resize((scene.width, scene.height))
    r.SetSettings(st)
    return r


@pytest.mark.parametrize("leaf_size", [3, 1])
def test_heightfield_full_size_per_path(heightfield, leaf_size):
    scene, o = heightfield
    W, H, ms = scene.width, scene.height, 16
    frames = scene.spp // ms
    st = tr.settings_for(scene, multi_sample=ms)
    r = renderer(scene, st, leaf_size)
    for _ in range(frames):
        r.RenderFrame(use_graph=True)
    stats = r.Statistics()
    assert stats["device_error"] == 0
    assert stats["sample_count"] == scene.spp
    buf = r.Buffers()
    acc = r.Accumulator().reshape(-1, 4)
    report = {}
    all_ok = []
    for name, rows in window_pixels(W).items():
        gpu_paths, orc_paths, gpu_acc, orc_acc, orc64 = [], [], [], [], []
        for first, count in rows:
            # per-path radiance of the last frame: path = pixel + sample * W * H
            rad = np.stack([r.read_device(buf["radiance"] + 16 * (first + s * W * H), np.float32, 4 * count)
                            .reshape(count, 4) for s in range(ms)])
            a32, p32, _ = o.render(scene.camera, st, W, H, frames=frames, first_pixel=first, pixel_count=count,
                                   want_paths=True)
            a64, _, _ = o.render(scene.camera, st, W, H, frames=frames, first_pixel=first, pixel_count=count,
                                 use_double=True)
            gpu_paths.append(rad[..., :3])
            orc_paths.append(p32[..., :3])
            gpu_acc.append(acc[first:first + count, :3] / acc[first:first + count, 3:4])
            orc_acc.append(a32[:, :3] / a32[:, 3:4])
            orc64.append(a64[:, :3] / a64[:, 3:4])
            np.testing.assert_array_equal(acc[first:first + count, 3], np.full(count, scene.spp, np.float32))
        g = np.concatenate(gpu_paths, 1).astype(np.float64)
        p = np.concatenate(orc_paths, 1)
        ok = close(g, p).all(-1)
        all_ok.append(ok.ravel())
        img_g, img_32, img_64 = (np.concatenate(x) for x in (gpu_acc, orc_acc, orc64))
        report[name] = dict(paths=float(ok.mean()), rmse_gpu_fp32=rel_rmse(img_g, img_32),
                            rmse_gpu_fp64=rel_rmse(img_g, img_64), rmse_fp32_fp64=rel_rmse(img_32, img_64),
                            mean=float(img_64.mean()))
    r.close()
    print(f"leaf size {leaf_size}: {report}")
    frac = float(np.concatenate(all_ok).mean())
    assert frac >= 0.995, f"per-path radiance within 1e-4 for {frac:.4f} of the window paths: {report}"
    for name, rep in report.items():
        assert rep["mean"] > 0, name
        assert rep["rmse_gpu_fp64"] <= 1.5 * rep["rmse_fp32_fp64"] + 1e-5, (name, rep)


def test_heightfield_full_size_hits_every_bounce(heightfield):
    """Stage by stage at full size (4 samples per pixel, 8.3 M paths in flight): the closest hits
    of every bounce's rays from the image rows of the windows (24 rows of 1920 pixels) against
    the oracle's traversal, bit-exact up to near ties; the rays of those rows that hit are
    exactly those the oracle sees hit."""
    scene, o = heightfield
    W, H, ms = scene.width, scene.height, 4
    st = tr.settings_for(scene, multi_sample=ms)
    r = renderer(scene, st)
    mask = np.zeros(W * H, bool)
    for _, y0 in WINDOWS.values():
        mask[y0 * W:(y0 + WIN_H) * W] = True
    r.BeginFrame()
    r.Generate()
    buf = r.Buffers()
    cap = buf["capacity"]

    def read_queue(k, n):
        planes = [r.read_device(buf["path_state"][k] + 16 * p * cap, np.float32, 4 * n).reshape(n, 4)
                  for p in range(2)]
        return planes

    checked = ties = 0
    for b in range(st.maxDepth):
        counters = r.read_device(buf["counters"], np.uint32, N_COUNTERS)
        count = cap if b == 0 else int(counters[b])
        if count == 0:
            break
        O, D = read_queue(0, count)
        paths = O[:, 3].view(np.uint32) >> 4
        sel = mask[paths % (W * H)]
        want = o.trace_closest(O[sel], D[sel], st.rayEpsilon)
        r.Extend(b)
        n_hit = int(r.read_device(buf["counters"], np.uint32, N_COUNTERS)[HIT_BASE + b])
        HO, HD = read_queue(1, n_hit)
        hits = r.read_device(buf["hits"], np.uint32, 4 * n_hit).reshape(n_hit, 4)
        hpaths = HO[:, 3].view(np.uint32) >> 4
        hsel = mask[hpaths % (W * H)]
        want_hit = want[:, 2] != 0xFFFFFFFF
        np.testing.assert_array_equal(np.sort(hpaths[hsel]), np.sort(paths[sel][want_hit]))
        # align the GPU's hit records with the oracle's by path index
        order_g = np.argsort(hpaths[hsel])
        order_o = np.argsort(paths[sel][want_hit])
        got = hits[hsel][order_g]
        exp = want[want_hit][order_o]
        go, gd = HO[hsel][order_g], HD[hsel][order_g]
        for i in np.where(~(got == exp).all(1))[0]:
            tg, tw = float(got[i, 3].view(np.float32)), float(exp[i, 3].view(np.float32))
            assert abs(tg - tw) <= 1e-6 * abs(tw), f"bounce {b}: gpu {got[i]} oracle {exp[i]}"
            near = o.ties(go[i], gd[i], st.rayEpsilon, tw, with_instances=True)
            assert (int(got[i, 1]), int(got[i, 2])) in near, f"bounce {b}: {got[i]} is no near tie of {exp[i]}"
            ties += 1
        checked += int(want_hit.sum())
        r.Shade(b)
        r.Connect(b)
    stats = r.Statistics()
    r.close()
    assert stats["device_error"] == 0
    print(f"hits checked {checked}, near ties {ties}")
    assert checked > 100_000 and ties <= checked // 1000


def test_cornell_full_size_every_path():
    """The closed box at its stated size: 256 x 256, 16 spp in one frame, 5 bounces, no RR."""
    scene = tr.cornell_box()
    assert (scene.width, scene.height, scene.spp, scene.max_depth) == (256, 256, 16, 5)
    assert scene.rr_start >= scene.max_depth  # no Russian roulette
    st = tr.settings_for(scene, multi_sample=16)
    r = renderer(scene, st)
    r.RenderFrame(use_graph=True)
    stats = r.Statistics()
    buf = r.Buffers()
    n = buf["capacity"]
    rad = r.read_device(buf["radiance"], np.float32, 4 * n).reshape(16, 256 * 256, 4)
    img = r.ColorBuffer().reshape(-1, 4)
    r.close()
    assert stats["device_error"] == 0
    o = Oracle(scene)
    a32, p32, counts = o.render(scene.camera, st, 256, 256, want_paths=True)
    a64, _, _ = o.render(scene.camera, st, 256, 256, use_double=True)
    ok = close(rad[..., :3].astype(np.float64), p32[..., :3]).all(-1)
    img32, img64 = a32[:, :3] / a32[:, 3:4], a64[:, :3] / a64[:, 3:4]
    g = img[:, :3].astype(np.float64)
    rep = dict(paths=float(ok.mean()), rmse_gpu_fp32=rel_rmse(g, img32), rmse_gpu_fp64=rel_rmse(g, img64),
               rmse_fp32_fp64=rel_rmse(img32, img64))
    print(f"cornell 256x256x16: {rep}")
    assert ok.mean() >= 0.995, rep
    assert rep["rmse_gpu_fp64"] <= 1.5 * rep["rmse_fp32_fp64"] + 1e-5, rep
    assert abs(stats["path_count"] - sum(counts)) <= 0.002 * sum(counts)
