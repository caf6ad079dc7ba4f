"""The path-replay adjoint on the CPU oracle (FP64): closure-value derivatives
against finite differences of the value, and the whole-path gradient against
central finite differences of the rendered loss for every parameter whose
change leaves the sampled paths unchanged (base colours, emission)."""
import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle

W = H = 12


def quantized(scene):
    """Material values exactly representable in fp16 (the upload rounds to fp16)."""
    m = scene.materials.copy()
    for f in ("diffuse", "emissive", "metallic", "roughness", "specular", "subsurface", "sheen", "clearcoat"):
        m[f] = m[f].astype(np.float16).astype(np.float32)
    scene.materials = m
    return scene


def test_closure_value_derivatives_match_finite_differences():
    scene = quantized(tr.cornell_box(width=W, height=H, wall_closure=tr.TR_CLOSURE_DISNEY))
    rng = np.random.default_rng(3)
    mats = scene.materials.copy()
    mats["roughness"] = rng.uniform(0.2, 0.9, len(mats)).astype(np.float16).astype(np.float32)
    mats["metallic"] = rng.uniform(0.1, 0.9, len(mats)).astype(np.float16).astype(np.float32)
    mats["specular"] = rng.uniform(0.1, 0.9, len(mats)).astype(np.float16).astype(np.float32)
    scene.materials = mats
    h = 2.0 ** -9
    names = [("diffuse", 0), ("diffuse", 1), ("diffuse", 2), ("roughness", None), ("metallic", None),
             ("specular", None)]
    for trial in range(20):
        m = int(rng.integers(0, 5))
        wo = rng.normal(size=3)
        wo[2] = abs(wo[2]) + 0.2
        wo /= np.linalg.norm(wo)
        wi = rng.normal(size=3)
        wi[2] = abs(wi[2]) + 0.2
        wi /= np.linalg.norm(wi)
        g = Oracle(scene).closure_value_grad(m, wo.astype(np.float32), wi.astype(np.float32))
        for p, (field, c) in enumerate(names):
            vals = []
            for sgn in (1, -1):
                mm = scene.materials.copy()
                if c is None:
                    mm[m][field] += sgn * h
                else:
                    mm[m][field][c] += sgn * h
                s2 = tr.Scene(scene.name, scene.positions, scene.normals, scene.texcoords, scene.indices,
                              scene.material_indices, mm)
                vals.append(Oracle(s2).closure_value_grad(m, wo.astype(np.float32), wi.astype(np.float32))[:, 0])
            fd = (vals[0] - vals[1]) / (2 * h)
            np.testing.assert_allclose(g[:, 1 + p], fd, rtol=2e-3, atol=1e-6,
                                       err_msg=f"material {m} param {p} trial {trial}")


def _loss_grad_check(scene, params):
    st = tr.settings_for(scene, multi_sample=8)
    st.maxColor = 1e30  # the firefly clamp is not differentiated (its scale is held fixed)
    rng = np.random.default_rng(0)
    w = rng.uniform(-1, 1, (H * W, 4)).astype(np.float32)
    w[:, 3] = 0

    def loss(mats):
        s2 = tr.Scene(scene.name, scene.positions, scene.normals, scene.texcoords, scene.indices,
                      scene.material_indices, mats)
        acc, _, _ = Oracle(s2).render(s2.camera, st, W, H, use_double=True)
        return float((acc[:, :3] / acc[:, 3:4] * w[:, :3]).sum())

    g = Oracle(scene).adjoint(scene.camera, st, W, H, 0, w, scale=1.0 / st.multiSample)
    for m, field, c, slot, h in params:
        mp, mm = scene.materials.copy(), scene.materials.copy()
        mp[m][field][c] += h
        mm[m][field][c] -= h
        fd = (loss(mp) - loss(mm)) / (2 * h)
        assert abs(fd - g[m, slot]) <= 1e-5 * max(1.0, abs(fd)), (m, field, c, fd, g[m, slot])


def test_path_gradient_base_colour_and_emission_match_fd():
    scene = quantized(tr.cornell_box(width=W, height=H))
    light = int(np.where(scene.materials["emissive"].sum(1) > 0)[0][0])
    params = [(m, "diffuse", c, c, 2.0 ** -8) for m in range(6) for c in range(3)]
    params += [(6, "diffuse", c, c, 2.0 ** -8) for c in range(3)]          # Disney conductor base colour
    params += [(light, "emissive", c, 6 + c, 2.0 ** -4) for c in range(3)]
    _loss_grad_check(scene, params)


def test_adjoint_rejects_reference_mode():
    scene = tr.cornell_box(width=4, height=4)
    st = tr.settings_for(scene, multi_sample=1, reference=True)
    with pytest.raises(RuntimeError):
        Oracle(scene).adjoint(scene.camera, st, 4, 4, 0, np.ones((16, 4), np.float32))
