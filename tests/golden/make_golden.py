"""Generates the golden fixtures of tests/golden from the reference's own code.

Runs where the reference sources are present (oracle/_ref/libtrref.so built by
oracle/build.py from the reference tree): the reference's closures
(Tracer/CUDA/GPU/Shade/BSDF/*.h), its random streams (thirdparty/CUDA/random.h)
and its raygen + path-tracing kernels (Tracer/Optix/GPU/optix.cu,
Tracer/CUDA/GPU/Shade/PathTracing.h), compiled as host C++, produce the
expected values; nothing here is written from memory.

    python tests/golden/make_golden.py              # every fixture
    python tests/golden/make_golden.py debug_modes  # only ref_debug_modes.npz
    python tests/golden/make_golden.py ray_picks    # only ref_ray_pick.npz
    python tests/golden/make_golden.py sky          # only ref_sky.npz
    python tests/golden/make_golden.py textures     # only ref_textures.npz
"""
from __future__ import annotations

import dataclasses
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import trayracer_gb300 as tr  # noqa: E402
from oracle import Reference, build  # noqa: E402
from trayracer_gb300.renderer import KernelSettings  # noqa: E402

OUT = Path(__file__).resolve().parent


def closure_inputs(n: int, seed: int) -> np.ndarray:
    """wo (z > 0.05), wi (any hemisphere), T, HitMaterial fields, r0, r1 (layout of ref_closure)."""
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 31), np.float32)

    def unit(k, zmin=None):
        v = rng.normal(size=(k, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        if zmin is not None:
            v[:, 2] = np.maximum(np.abs(v[:, 2]), zmin)
            v /= np.linalg.norm(v, axis=1, keepdims=True)
        return v.astype(np.float32)

    x[:, 0:3] = unit(n, 0.05)
    x[:, 3:6] = unit(n)
    x[:, 6:9] = rng.uniform(0.05, 1.0, (n, 3))
    q = x[:, 9:]
    diffuse = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    q[:, 0:3] = diffuse
    q[:, 3] = rng.uniform(0, 1, n)       # metallic
    q[:, 4:7] = 0                        # emissive
    q[:, 7] = np.where(rng.uniform(size=n) < 0.3, rng.uniform(0, 1, n), 0)  # subsurface
    # tint / luminance from CIE XYZ of the diffuse colour (CudaMaterial.h:155-183)
    d = diffuse
    X = np.maximum(0, np.float32(0.412453) * d[:, 0] + np.float32(0.357580) * d[:, 1] + np.float32(0.180423) * d[:, 2])
    Y = np.maximum(0, np.float32(0.212671) * d[:, 0] + np.float32(0.715160) * d[:, 1] + np.float32(0.072169) * d[:, 2])
    Z = np.maximum(0, np.float32(0.019334) * d[:, 0] + np.float32(0.119193) * d[:, 1] + np.float32(0.950227) * d[:, 2])
    Yn = np.where(Y > 0, Y, 1).astype(np.float32)
    xx, yy, zz = X / Yn, Y / Yn, Z / Yn
    tint = np.stack([
        np.maximum(0, np.float32(3.240479) * xx - np.float32(1.537150) * yy - np.float32(0.498535) * zz),
        np.maximum(0, np.float32(-0.969256) * xx + np.float32(1.875992) * yy + np.float32(0.041556) * zz),
        np.maximum(0, np.float32(0.055648) * xx - np.float32(0.204043) * yy + np.float32(1.057311) * zz),
    ], axis=1)
    q[:, 8:11] = np.where((Y > 0)[:, None], tint, 1)
    q[:, 11] = rng.uniform(0, 1, n)      # specular
    q[:, 12] = rng.uniform(0.02, 1, n)   # roughness
    q[:, 13] = rng.uniform(0, 1, n)      # specularTint
    q[:, 14] = np.where(rng.uniform(size=n) < 0.3, rng.uniform(-1, 1, n), 0)  # anisotropic
    q[:, 15] = np.where(rng.uniform(size=n) < 0.3, rng.uniform(0, 1, n), 0)   # sheen
    q[:, 16] = rng.uniform(0, 1, n)      # sheenTint
    q[:, 17] = np.where(rng.uniform(size=n) < 0.3, rng.uniform(0, 1, n), 0)   # clearcoat
    q[:, 18] = rng.uniform(0, 1, n)      # clearcoatGloss
    q[:, 19] = Y
    q[:, 20] = rng.uniform(0, 1, n)      # r0
    q[:, 21] = rng.uniform(0, 1, n)      # r1
    return x


def cornell_reference_frames(width=32, height=32, ms=1, seed=5, frames=2):
    """The reference's frame loop on the Cornell box (Lambert everywhere, as PathTracing.h:129)."""
    scene = tr.cornell_box(wall_closure=tr.TR_CLOSURE_LAMBERT, width=width, height=height)
    st = KernelSettings(multiSample=ms, maxDepth=scene.max_depth, seed=seed, rrStart=1,
                        flags=tr.TR_FLAG_REFERENCE_SAMPLING | tr._abi.TR_FLAG_REFERENCE_DRAW_RTL)
    ref = Reference(scene)
    acc = np.zeros((width * height, 4), np.float32)
    accs, exts, shs = [], [], []
    for f in range(frames):
        ext, sh = ref.render_frame(scene.camera, st, width, height, f * ms, acc)
        accs.append(acc.copy())
        exts.append(ext.copy())
        shs.append(sh.copy())
    # stage data of the first frame: primary rays + hits, and the shade of bounce 0
    acc0 = np.zeros((width * height, 4), np.float32)
    states, hits = ref.primary(scene.camera, st, width, height, 0, acc0)
    prim_states, prim_hits = states.copy(), hits.copy()
    shadow = np.zeros_like(states)
    n_ext, n_sh = ref.shade(scene.camera, st, width, height, 0, 0, width * height * ms, states, hits, shadow, acc0)
    return dict(
        digest=np.array(scene.digest()), width=width, height=height, ms=ms, seed=seed, frames=frames,
        acc=np.stack(accs), ext=np.stack(exts), sh=np.stack(shs),
        prim_states=prim_states, prim_hits=prim_hits,
        shade_states=states[:, :n_ext].copy(), shade_shadow=shadow[:, :n_sh].copy(), shade_acc=acc0,
    )


DEBUG_MODES = [(0, 0), (1, 0), (2, 0), (3, 0), (4, 0), (5, 3), (5, 4), (5, 6), (5, 7), (6, 0), (8, 0), (9, 0),
               (10, 0), (11, 0), (12, 0)]


def debug_mode_frames(width=40, height=30, seed=5, ao_dist=0.6, z_depth_max=3.0):
    """One frame of every other render mode (RenderModes 0-12 except 7; MaterialProperty with
    MaterialPropertyIds Diffuse, Emissive, Normal, Roughness) on the two-level Cornell box, by the
    reference's raygen programs and shade kernels (Tracer/CUDA/GPU/Shade/*.h)."""
    scene = tr.instanced_cornell(width=width, height=height)
    st = KernelSettings(multiSample=1, maxDepth=2, seed=seed, rrStart=1,
                        flags=tr.TR_FLAG_REFERENCE_SAMPLING | tr._abi.TR_FLAG_REFERENCE_DRAW_RTL)
    ref = Reference(scene)
    out = dict(digest=np.array(scene.digest()), width=width, height=height, seed=seed, ao_dist=ao_dist,
               z_depth_max=z_depth_max, modes=np.array(DEBUG_MODES, np.uint32))
    for mode, flags in DEBUG_MODES:
        Reference.set_render_mode(mode, flags, ao_dist, z_depth_max)
        acc = np.zeros((width * height, 4), np.float32)
        ref.render_frame(scene.camera, st, width, height, 0, acc)
        out[f"mode_{mode}_{flags}"] = acc
    Reference.set_render_mode(7)
    return out


PICK_CAMERA_FIELDS = ("position", "target", "up", "fov", "aperture", "distortion", "focal_dist", "bokeh_side_count",
                      "bokeh_rotation")


def pick_cases():
    """(name, scene, camera) triples of the ray-pick fixture: the Cornell box, the two-level Cornell
    box and a heightfield seen through a six-bladed aperture with lens distortion (misses included)."""
    hf = tr.heightfield(n=16, width=32, height=32)
    lens = dataclasses.replace(hf.camera, aperture=0.05, focal_dist=12.0, bokeh_side_count=6, bokeh_rotation=0.3,
                               distortion=0.1)
    return [("cornell", tr.cornell_box(width=40, height=30), None),
            ("instanced_cornell", tr.instanced_cornell(width=40, height=30), None),
            ("heightfield_lens", hf, lens)]


def pick_pixels(w, h):
    """Every third column and second row plus a margin of two pixels outside the image."""
    return np.array([(x, y) for x in range(-2, w + 2, 3) for y in range(-2, h + 3, 2)], np.int32)


def ray_picks():
    """DeviceRenderer::PickRay results (RayPickResult words, as uint32) by the reference's RayPick
    raygen (optix.cu:345-377) compiled as host C++."""
    out = {}
    st = KernelSettings(flags=tr.TR_FLAG_REFERENCE_SAMPLING | tr._abi.TR_FLAG_REFERENCE_DRAW_RTL)
    for name, scene, cam in pick_cases():
        cam = cam or scene.camera
        ref = Reference(scene)
        px = pick_pixels(scene.width, scene.height)
        res = np.stack([ref.pick_ray(cam, st, scene.width, scene.height, x, y) for x, y in px])
        out[f"{name}_digest"] = np.array(scene.digest())
        out[f"{name}_camera"] = np.array([float(np.asarray(getattr(cam, f), np.float64).ravel()[i])
                                          for f in PICK_CAMERA_FIELDS
                                          for i in range(np.asarray(getattr(cam, f)).size)], np.float64)
        out[f"{name}_size"] = np.array([scene.width, scene.height], np.int32)
        out[f"{name}_pixels"] = px
        out[f"{name}_result"] = res.view(np.uint32)
    return out


SKY_CASES = {
    "sun_high": dict(sunDir=(0.2, 0.9, 0.4)),
    "sun_low": dict(sunDir=(0.4, 0.15, 0.8), turbidity=6.5, sunAngularDiameter=300.0),
    "sun_set": dict(sunDir=(0.0, -0.2, 1.0), drawSun=False),
}


def sky_frames(width=32, height=24, seed=3, max_depth=4):
    """One frame of the outdoor heightfield (Lambert) under three skies by the reference's
    kernels (SampleSky, CudaSky.h:105-156, on every path that leaves the scene)."""
    scene = tr.outdoor_heightfield(width=width, height=height, lambert=True)
    st = KernelSettings(multiSample=1, maxDepth=max_depth, seed=seed, rrStart=1,
                        flags=tr.TR_FLAG_REFERENCE_SAMPLING | tr._abi.TR_FLAG_REFERENCE_DRAW_RTL)
    out = dict(digest=np.array(scene.digest()), width=width, height=height, seed=seed, max_depth=max_depth)
    for name, kw in SKY_CASES.items():
        ref = Reference(scene)
        ref.set_sky(tr.SkySettings(**kw))
        acc = np.zeros((width * height, 4), np.float32)
        ref.render_frame(scene.camera, st, width, height, 0, acc)
        out[f"{name}_acc"] = acc
    return out


TEXTURE_MODES = [(5, 3), (5, 5), (5, 6), (5, 7), (8, 0)]


def texture_frames(width=32, height=24, seed=11):
    """The textured Cornell box (Lambert) by the reference's kernels with their tex2D fetches
    served by the oracle's restatement of the texture unit's bilinear filter: one path-traced
    frame (reference sampling) and the material-property / shading-normal images of
    TEXTURE_MODES."""
    scene = tr.textured_cornell(width=width, height=height, wall_closure=tr.TR_CLOSURE_LAMBERT)
    st = KernelSettings(multiSample=1, maxDepth=5, seed=seed, rrStart=1,
                        flags=tr.TR_FLAG_REFERENCE_SAMPLING | tr._abi.TR_FLAG_REFERENCE_DRAW_RTL)
    out = dict(digest=np.array(scene.digest()), width=width, height=height, seed=seed,
               modes=np.array(TEXTURE_MODES, np.uint32))
    ref = Reference(scene)
    acc = np.zeros((width * height, 4), np.float32)
    ref.render_frame(scene.camera, st, width, height, 0, acc)
    out["frame"] = acc
    for mode, flags in TEXTURE_MODES:
        Reference.set_render_mode(mode, flags, 1.0, 1.0)
        acc = np.zeros((width * height, 4), np.float32)
        ref.render_frame(scene.camera, st, width, height, 0, acc)
        out[f"mode_{mode}_{flags}"] = acc
    Reference.set_render_mode(7)
    return out


def main():
    single = {"debug_modes": ("ref_debug_modes.npz", debug_mode_frames), "ray_picks": ("ref_ray_pick.npz", ray_picks),
              "sky": ("ref_sky.npz", sky_frames), "textures": ("ref_textures.npz", texture_frames)}
    if len(sys.argv) == 2 and sys.argv[1] in single:
        build.build_oracle()
        if build.build_reference() is None:
            raise SystemExit("reference sources not found")
        name, make = single[sys.argv[1]]
        np.savez_compressed(OUT / name, **make())
        return
    build.build_oracle()
    if build.build_reference() is None:
        raise SystemExit("reference sources not found: the golden fixtures come from the reference's own code")
    # random streams
    pairs = np.array([[0, 0], [1, 2], [5, 0], [123456, 7], [0xFFFFFFFF, 3], [77, 1 << 20]], np.uint32)
    draws = np.stack([Reference.rng(int(a), int(b), 16) for a, b in pairs])
    np.savez_compressed(OUT / "ref_rng.npz", pairs=pairs, draws=draws)
    # closures
    out = {}
    for ctype, name in ((tr.TR_CLOSURE_LAMBERT, "lambert"), (tr.TR_CLOSURE_DIFFUSE, "diffuse"),
                        (tr.TR_CLOSURE_DISNEY, "disney")):
        x = closure_inputs(1500, seed=11 + ctype)
        out[f"{name}_in"] = x
        out[f"{name}_out"] = Reference.closure(ctype, x)
    np.savez_compressed(OUT / "ref_closures.npz", **out)
    # frames
    np.savez_compressed(OUT / "ref_cornell_32x32_ms1.npz", **cornell_reference_frames(ms=1))
    np.savez_compressed(OUT / "ref_cornell_24x16_ms2.npz", **cornell_reference_frames(24, 16, ms=2, seed=9))
    # the other render modes
    np.savez_compressed(OUT / "ref_debug_modes.npz", **debug_mode_frames())
    # ray picks
    np.savez_compressed(OUT / "ref_ray_pick.npz", **ray_picks())
    # the sky
    np.savez_compressed(OUT / "ref_sky.npz", **sky_frames())
    # textures
    np.savez_compressed(OUT / "ref_textures.npz", **texture_frames())
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
