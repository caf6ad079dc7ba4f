"""GPU parity: every stage of the wavefront against the CPU oracle, on the
same inputs, through the C ABI (libtrayracer.so).

Tolerances (the oracle runs the same fp32 algorithm; the GPU contracts
multiply-adds and uses its own transcendental functions):
  hits       bit-exact primitive, t and 16-bit barycentrics, except logged
             near ties (|dt| <= 1e-6 t) between coplanar or edge-sharing triangles;
  rays       |a - b| <= 1e-4 * max(1, |b|) per component;
  radiance   per-path within 1e-4 relative (atol 1e-6), for all but a
             logged fraction of paths whose discrete decisions (Russian roulette,
             NEE gate, lobe choice) flipped on a last-bit difference.
"""
import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle
from trayracer_gb300._abi import TR_FLAG_REFERENCE_DRAW_RTL
from trayracer_gb300.renderer import KernelSettings

pytestmark = pytest.mark.gpu

RTOL = 1e-4
N_COUNTERS = 5 * 17  # extend, shadow, extend cursor, connect cursor, hit queue length; per bounce
HIT_BASE = 4 * 17


def close(a, b, rtol=RTOL, atol=1e-6):
    return np.abs(a - b) <= rtol * np.maximum(1.0, np.abs(b)) + atol


def make_renderer(scene, settings):
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene)
    r.SetCamera(scene.camera)
    r.Resize((scene.width, scene.height))
    r.SetSettings(settings)
    return r


def read_state(r, buf, k, n):
    cap = buf["capacity"]
    a = r.read_device(buf["path_state"][k], np.float32, 3 * cap * 4).reshape(3, cap, 4)
    return a[:, :n].copy()


def frac(ok):
    """Fraction of True entries; 1 for an empty selection (a bounce with no rays of that kind)."""
    return float(ok.mean()) if ok.size else 1.0


def within_conditioning(gpu, o32, o64, sens):
    """|gpu - fp64| <= 1e-4 max(1, |fp64|) + 4 |fp32 oracle - fp64| + sens, element-wise, where
    sens is how far the FP64 result moves when the inputs move by a few ulps (see
    shade_sensitivity): a backward-stable fp32 evaluation errs by about that much."""
    return np.abs(gpu - o64) <= RTOL * np.maximum(1.0, np.abs(o64)) + 4.0 * np.abs(o32 - o64) + sens + 1e-6


def shade_sensitivity(o, st, b, W, H, state, hits, ext64, sh64):
    """Largest change of the FP64 shading outputs when the ray directions move by 2^-21
    relative (about 4 ulps, both signs, alternating per component). Near-specular GGX lobes
    (roughness <= 0.1) turn such input changes into output changes far above 1e-4."""
    sens_e = np.zeros(ext64.shape, np.float64)
    sens_s = np.zeros(sh64.shape, np.float64)
    for sgn in (1.0, -1.0):
        pat = np.array([1.0, -1.0, 1.0]) * sgn
        D = state[1].copy()
        D[:, :3] = (D[:, :3].astype(np.float64) * (1.0 + pat * 2.0 ** -21)).astype(np.float32)
        e, _, sh, _, _ = o.shade(st, b, 0, W, H, state[0], D, state[2], hits, fp64=True)
        with np.errstate(invalid="ignore"):
            # entries without an extend / shadow ray may hold NaN: fmax keeps the other value
            sens_e = np.fmax(sens_e, np.abs(e.astype(np.float64) - ext64))
            sens_s = np.fmax(sens_s, np.abs(sh.astype(np.float64) - sh64))
    return sens_e, sens_s


def hit_materials(scene, insts, prims):
    """Material index of hits (instance, triangle of the instance's mesh)."""
    if getattr(scene, "instances", None) is None:
        return scene.material_indices[prims]
    out = np.empty(len(prims), np.int64)
    for k, (i, p) in enumerate(zip(insts, prims)):
        mesh = scene.instances[int(i)][0]
        out[k] = int(scene.mesh_material_offsets[mesh]) + int(scene.meshes[mesh]["material_indices"][int(p)])
    return out


def pdf_tolerance(scene, insts, prims):
    """Relative tolerance of the extend pdf (T.w) of each shaded hit. The GGX distribution is
    evaluated from tan^2(theta) = (1 - cos^2 theta) / cos^2 theta of the sampled microfacet
    normal (Shade/BSDF/Microfacet.h:143-151); cos theta is within a few fp32 ulps, so near the
    peak of a lobe of width alpha the factor 1 + tan^2(theta) / alpha^2 and hence the pdf are only
    defined to about (ulps * 2^-23) / alpha^2 relative, alpha = max(0.001, roughness^2)
    (Microfacet.h:33-36). Allowed: 1e-4 + 32 * 2^-23 / alpha^2 for Disney materials."""
    m = scene.materials[hit_materials(scene, insts, prims)]
    alpha = np.maximum(0.001, m["roughness"].astype(np.float64) ** 2)
    return np.where(m["closure"] == tr.TR_CLOSURE_DISNEY, RTOL + 32 * 2.0 ** -23 / alpha ** 2, RTOL)


def check_hits(o, O, D, got, eps):
    want = o.trace_closest(O, D, eps)
    same = (got == want).all(axis=1)
    ties = 0
    for i in np.where(~same)[0]:
        tg = float(got[i, 3].view(np.float32))
        tw = float(want[i, 3].view(np.float32))
        assert abs(tg - tw) <= 1e-6 * abs(tw), f"ray {i}: gpu {got[i]} oracle {want[i]}"
        near = o.ties(O[i], D[i], eps, tw, with_instances=True)
        assert (int(got[i, 1]), int(got[i, 2])) in near, f"ray {i}: {got[i]} is no near tie of {want[i]}"
        ties += 1
    return ties


SCENES = {
    "cornell_counter": lambda: (tr.cornell_box(width=48, height=40), dict(ms=2, reference=False)),
    "cornell_reference": lambda: (tr.cornell_box(width=40, height=32), dict(ms=2, reference=True)),
    "heightfield_counter": lambda: (tr.heightfield(n=128, width=64, height=36, rr_start=2),
                                    dict(ms=2, reference=False)),
    "instanced_counter": lambda: (tr.instanced_cornell(width=48, height=40), dict(ms=2, reference=False)),
    "instanced_reference": lambda: (tr.instanced_cornell(width=40, height=32), dict(ms=2, reference=True)),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_stagewise_parity(name):
    scene, kw = SCENES[name]()
    st = tr.settings_for(scene, multi_sample=kw["ms"], reference=kw["reference"])
    o = Oracle(scene)
    r = make_renderer(scene, st)
    W, H = scene.width, scene.height
    r.BeginFrame()
    r.Generate()
    buf = r.Buffers()
    n = buf["capacity"]
    s0 = read_state(r, buf, 0, n)
    O, D, T = o.generate(scene.camera, st, W, H, 0, 0, n)
    np.testing.assert_array_equal(s0[0][:, 3].view(np.uint32), O[:, 3].view(np.uint32))
    assert close(s0[0][:, :3], O[:, :3]).all()
    assert close(s0[1][:, :3], D[:, :3]).all()
    assert close(s0[2], T).all()

    radiance = np.zeros((n, 4), np.float32)
    total_ties = 0
    flipped = 0
    for b in range(st.maxDepth):
        counters = r.read_device(buf["counters"], np.uint32, N_COUNTERS)
        count = n if b == 0 else int(counters[b])
        if count == 0:
            break
        queue = read_state(r, buf, 0, count)
        r.Extend(b)
        # the hit queue holds exactly the rays the oracle sees hit something
        counters = r.read_device(buf["counters"], np.uint32, N_COUNTERS)
        n_hit = int(counters[HIT_BASE + b])
        state = read_state(r, buf, 1, n_hit)
        want_hit = o.trace_closest(queue[0], queue[1], st.rayEpsilon)[:, 2] != 0xFFFFFFFF
        q_paths = queue[0][:, 3].view(np.uint32) >> 4
        np.testing.assert_array_equal(np.sort(state[0][:, 3].view(np.uint32) >> 4), np.sort(q_paths[want_hit]))
        hits = r.read_device(buf["hits"], np.uint32, n_hit * 4).reshape(n_hit, 4)
        total_ties += check_hits(o, state[0], state[1], hits, st.rayEpsilon)

        r.Shade(b)
        counters = r.read_device(buf["counters"], np.uint32, N_COUNTERS)
        n_ext, n_sh = int(counters[b + 1]), int(counters[17 + b])
        ext_gpu = read_state(r, buf, 0, n_ext)
        sh_gpu = r.read_device(buf["shadow"], np.float32, 3 * n * 4).reshape(3, n, 4)[:, :n_sh]
        rad_gpu = r.read_device(buf["radiance"], np.float32, n * 4).reshape(n, 4)
        ext, ev, sh, sv, add = o.shade(st, b, 0, W, H, state[0], state[1], state[2], hits)
        ext64, _, sh64, _, _ = o.shade(st, b, 0, W, H, state[0], state[1], state[2], hits, fp64=True)
        sens_e, sens_s = shade_sensitivity(o, st, b, W, H, state, hits, ext64, sh64)
        path = state[0][:, 3].view(np.uint32) >> 4

        # extend rays, matched by path index
        gpu_ext_paths = ext_gpu[0][:, 3].view(np.uint32) >> 4
        orc_ext_paths = path[ev]
        sym = np.setxor1d(gpu_ext_paths, orc_ext_paths)
        flipped += sym.size
        assert sym.size <= max(2, count // 500), f"bounce {b}: {sym.size} extend decisions differ"
        common = np.intersect1d(gpu_ext_paths, orc_ext_paths)
        gi = np.argsort(gpu_ext_paths)[np.searchsorted(np.sort(gpu_ext_paths), common)]
        oe = ext[ev]
        oi = np.argsort(orc_ext_paths)[np.searchsorted(np.sort(orc_ext_paths), common)]
        np.testing.assert_array_equal(ext_gpu[0][gi, 3].view(np.uint32), oe[oi, 0, 3].view(np.uint32))
        ok = close(ext_gpu[0][gi, :3], oe[oi, 0, :3]).all(1) & close(ext_gpu[1][gi, :3], oe[oi, 1, :3]).all(1)
        assert frac(ok) >= 0.998, f"bounce {b}: extend ray origins/directions agree for {frac(ok):.4f}"
        # throughput and pdf: near-specular GGX lobes are ill-conditioned in fp32, so the GPU is
        # held to the FP64 shading of the same inputs within 1e-4, plus a few times the fp32
        # oracle's own distance from it, plus the FP64 result's change under few-ulp input changes
        oe64 = ext64[ev]
        okt = within_conditioning(ext_gpu[2][gi, :3], oe[oi, 2, :3], oe64[oi, 2, :3], sens_e[ev][oi, 2, :3]).all(1)
        assert frac(okt) >= 0.998, f"bounce {b}: extend throughputs agree for {frac(okt):.4f}"
        pdf64 = oe64[oi, 2, 3].astype(np.float64)
        okp = np.abs(ext_gpu[2][gi, 3] - pdf64) <= pdf_tolerance(scene, hits[ev][oi, 1], hits[ev][oi, 2]) * np.maximum(1.0, pdf64)
        assert frac(okp) >= 0.998, f"bounce {b}: extend pdfs agree for {frac(okp):.4f}"

        # shadow rays, matched by path index
        gpu_sh_paths = sh_gpu[0][:, 3].view(np.uint32)
        orc_sh_paths = path[sv]
        sym = np.setxor1d(gpu_sh_paths, orc_sh_paths)
        flipped += sym.size
        assert sym.size <= max(2, count // 500), f"bounce {b}: {sym.size} NEE decisions differ"
        common = np.intersect1d(gpu_sh_paths, orc_sh_paths)
        gi = np.argsort(gpu_sh_paths)[np.searchsorted(np.sort(gpu_sh_paths), common)]
        osh = sh[sv]
        oi = np.argsort(orc_sh_paths)[np.searchsorted(np.sort(orc_sh_paths), common)]
        ok = close(sh_gpu[0][gi, :3], osh[oi, 0, :3]).all(1) & close(sh_gpu[1][gi], osh[oi, 1]).all(1) \
            & within_conditioning(sh_gpu[2][gi, :3], osh[oi, 2, :3], sh64[sv][oi, 2, :3],
                                  sens_s[sv][oi, 2, :3]).all(1)
        assert frac(ok) >= 0.998, f"bounce {b}: shadow rays agree for {frac(ok):.4f}"

        # radiance added by shade
        want_rad = radiance.copy()
        np.add.at(want_rad, path, add)
        okr = close(rad_gpu[:, :3], want_rad[:, :3], rtol=1e-4).all(1)
        assert frac(okr) >= 0.999, f"bounce {b}: shade radiance agrees for {frac(okr):.4f}"

        # connect: unoccluded shadow rays add their throughput
        r.Connect(b)
        rad_after = r.read_device(buf["radiance"], np.float32, n * 4).reshape(n, 4)
        if n_sh:
            occ = o.trace_any(sh_gpu[0], sh_gpu[1], st.rayEpsilon).astype(bool)
            want2 = rad_gpu.copy()
            vis = ~occ
            np.add.at(want2, gpu_sh_paths[vis], sh_gpu[2][vis])
            okc = close(rad_after[:, :3], want2[:, :3], rtol=1e-5).all(1)
            assert frac(okc) >= 0.9995, f"bounce {b}: connect agrees for {frac(okc):.5f}"
        radiance = rad_after
    print(f"{name}: near ties {total_ties}, flipped decisions {flipped}")
    r.close()


@pytest.mark.parametrize("reference,two_level", [(False, False), (True, False), (False, True), (True, True)])
def test_frame_parity_per_path(reference, two_level):
    scene = tr.instanced_cornell(width=64, height=48) if two_level else tr.cornell_box(width=64, height=48)
    st = tr.settings_for(scene, multi_sample=4, reference=reference)
    r = make_renderer(scene, st)
    r.RenderFrame()
    buf = r.Buffers()
    n = buf["capacity"]
    rad = r.read_device(buf["radiance"], np.float32, n * 4).reshape(st.multiSample, scene.height * scene.width, 4)
    img = r.ColorBuffer()
    stats = r.Statistics()
    r.close()
    assert stats["device_error"] == 0
    acc, paths, counts = Oracle(scene).render(scene.camera, st, scene.width, scene.height, want_paths=True)
    ok = close(rad[..., :3].astype(np.float64), paths[..., :3], rtol=1e-4).all(-1)
    assert ok.mean() >= 0.995, ok.mean()
    ref_img = (acc[:, :3] / acc[:, 3:4]).reshape(scene.height, scene.width, 3)
    rel_rmse = np.sqrt(np.mean((img[..., :3] - ref_img) ** 2)) / np.sqrt(np.mean(ref_img ** 2))
    assert rel_rmse < 1e-2, rel_rmse
    # ray counts of the wavefront and of the depth-first oracle agree up to flipped decisions
    assert abs(stats["path_count"] - sum(counts)) <= 0.002 * sum(counts)


def test_image_rmse_against_fp64_oracle():
    """The GPU image against the FP64 oracle's with the same sample keys: no further from it than
    the fp32 oracle is (the residual is fp32 against fp64 path divergence, which falls as
    1/sqrt(spp)), and within 1e-3 relative RMSE at 16 spp."""
    scene = tr.cornell_box(width=48, height=48)
    st = tr.settings_for(scene, multi_sample=8)
    r = make_renderer(scene, st)
    for _ in range(2):
        r.RenderFrame()
    img = r.ColorBuffer()
    r.close()
    o = Oracle(scene)
    acc64, _, _ = o.render(scene.camera, st, 48, 48, frames=2, use_double=True)
    acc32, _, _ = o.render(scene.camera, st, 48, 48, frames=2)
    ref = (acc64[:, :3] / acc64[:, 3:4]).reshape(48, 48, 3)
    ref32 = (acc32[:, :3] / acc32[:, 3:4]).reshape(48, 48, 3)

    def rel(a, b):
        return np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2))

    rel_rmse, rel32 = rel(img[..., :3], ref), rel(ref32, ref)
    print(f"relative image RMSE vs FP64 oracle: GPU {rel_rmse:.3e}, fp32 oracle {rel32:.3e}")
    assert rel_rmse <= 1.5 * rel32 + 1e-5, (rel_rmse, rel32)
    assert rel_rmse < 1e-3, rel_rmse


@pytest.mark.parametrize("fixture", ["ref_cornell_32x32_ms1.npz", "ref_cornell_24x16_ms2.npz"])
def test_gpu_against_reference_golden(fixture):
    """The GPU kernels in reference mode (right-to-left draws, Lambert closures)
    against the accumulator the reference's own kernels produced."""
    from pathlib import Path

    g = np.load(Path(__file__).resolve().parent / "golden" / fixture)
    w, h, ms, seed = int(g["width"]), int(g["height"]), int(g["ms"]), int(g["seed"])
    scene = tr.cornell_box(wall_closure=tr.TR_CLOSURE_LAMBERT, width=w, height=h)
    assert scene.digest() == str(g["digest"])
    st = KernelSettings(multiSample=ms, maxDepth=5, seed=seed, rrStart=1,
                        flags=tr.TR_FLAG_REFERENCE_SAMPLING | TR_FLAG_REFERENCE_DRAW_RTL)
    r = make_renderer(scene, st)
    # stage check on the first frame: primary rays and hits
    r.BeginFrame()
    r.Generate()
    buf = r.Buffers()
    n = buf["capacity"]
    s0 = read_state(r, buf, 0, n)
    ps = g["prim_states"]
    assert close(s0[0][:, :3], ps[0][:, :3]).all() and close(s0[1][:, :3], ps[1][:, :3]).all()
    r.Extend(0)
    n_hit = int(r.read_device(buf["counters"], np.uint32, N_COUNTERS)[HIT_BASE])
    hits = r.read_device(buf["hits"], np.uint32, n_hit * 4).reshape(n_hit, 4)
    paths = read_state(r, buf, 1, n_hit)[0][:, 3].view(np.uint32) >> 4
    # the reference indexes hits by path (misses carry primIx ~0); the hit queue by slot
    prim = np.full(n, 0xFFFFFFFF, np.uint32)
    prim[paths] = hits[:, 2]
    match = (prim == g["prim_hits"][:, 2]).mean()
    assert match >= 0.995, match
    r.Reset()
    for f in range(int(g["frames"])):
        r.RenderFrame()
    acc = r.Accumulator().reshape(-1, 4)
    r.close()
    want = g["acc"][-1]
    ok = close(acc[:, :3], want[:, :3], rtol=1e-4).all(1)
    assert ok.mean() >= 0.99, ok.mean()
    np.testing.assert_array_equal(acc[:, 3], want[:, 3])
