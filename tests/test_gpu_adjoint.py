"""The GPU path-replay adjoint: against the FP64 oracle's gradient of the same
estimator (relative 1e-4; with Russian roulette and 12 bounces too), against
central finite differences of GPU renders (parameters whose change leaves the
sampled paths fixed: within 1e-2; roughness, metallic and specular, which move
the sampled directions: statistically over seeds), on the differentiation
configuration (512 x 512, 32 spp, L2 loss against a perturbed target), and
through the libtorch autograd function. Firefly clamp off (its scale is not
differentiated)."""
import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle
from trayracer_gb300.renderer import KernelSettings

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def diff_scene(w, h):
    scene = tr.cornell_box(width=w, height=h, wall_closure=tr.TR_CLOSURE_DISNEY, max_depth=6)
    m = scene.materials.copy()
    rng = np.random.default_rng(5)
    disney = m["closure"] == tr.TR_CLOSURE_DISNEY
    m["roughness"][disney] = rng.uniform(0.3, 0.9, disney.sum())
    m["specular"][disney] = rng.uniform(0.2, 0.8, disney.sum())
    m["metallic"][disney & (m["metallic"] == 0)] = rng.uniform(0.0, 0.3, (disney & (m["metallic"] == 0)).sum())
    for f in ("diffuse", "emissive", "metallic", "roughness", "specular"):
        m[f] = m[f].astype(np.float16).astype(np.float32)
    scene.materials = m
    return scene


def settings(spp, depth=6, rr_start=1 << 30):
    return KernelSettings(multiSample=spp, maxDepth=depth, seed=3, rrStart=rr_start, maxColor=1e30)


def rel_difference(g, want):
    """Relative L2 difference over the entries above 1 % of the largest."""
    big = np.abs(want) > 1e-2 * np.abs(want).max()
    return float(np.linalg.norm(g[big] - want[big]) / np.linalg.norm(want[big]))


def gpu_adjoint(scene, st, weights):
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene)
    r.SetCamera(scene.camera)
    r.Resize((scene.width, scene.height))
    r.SetSettings(st)
    r.RenderFrame()
    pg = torch.from_numpy(weights.reshape(scene.height, scene.width, 4)).cuda()
    grad = torch.zeros((scene.materials.shape[0], 9), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    r.AdjointFrame(pg.data_ptr(), 1.0 / st.multiSample, grad.data_ptr())
    torch.cuda.synchronize()
    out = grad.cpu().numpy()
    r.close()
    return out


def test_gpu_adjoint_matches_fp64_oracle():
    scene = diff_scene(32, 32)
    st = settings(16)
    rng = np.random.default_rng(1)
    w = rng.uniform(-1, 1, (32 * 32, 4)).astype(np.float32)
    w[:, 3] = 0
    g_gpu = gpu_adjoint(scene, st, w)
    g_cpu = Oracle(scene).adjoint(scene.camera, st, 32, 32, 0, w, scale=1.0 / st.multiSample, use_double=True)
    rel = rel_difference(g_gpu, g_cpu)
    print(f"relative gradient difference GPU vs FP64 oracle: {rel:.2e}")
    assert rel < 1e-4, rel


def test_gpu_adjoint_with_russian_roulette_deep_paths():
    """12 bounces with Russian roulette from bounce 3 (the large configuration's depth): the
    replay carries each path's remaining radiance forward, so no per-bounce state is kept
    however deep the path; the survival factor 1/rr (Shade/PathTracing.h:149-155) is held fixed
    like the sampling pdfs (detached), which keeps the gradient estimator unbiased:
    E[d(g)/rr 1{u < rr}] = d(g) for any rr. Against the oracle's adjoint of the same estimator
    (fp32: the same Russian-roulette decisions; FP64: decisions may flip on a last-bit
    difference)."""
    scene = diff_scene(32, 32)
    st = settings(16, depth=12, rr_start=3)
    rng = np.random.default_rng(3)
    w = rng.uniform(-1, 1, (32 * 32, 4)).astype(np.float32)
    w[:, 3] = 0
    g_gpu = gpu_adjoint(scene, st, w)
    o = Oracle(scene)
    g32 = o.adjoint(scene.camera, st, 32, 32, 0, w, scale=1.0 / st.multiSample, use_double=False)
    g64 = o.adjoint(scene.camera, st, 32, 32, 0, w, scale=1.0 / st.multiSample, use_double=True)
    rel32, rel64, rel_o = rel_difference(g_gpu, g32), rel_difference(g_gpu, g64), rel_difference(g32, g64)
    print(f"RR adjoint, 12 bounces: GPU vs fp32 oracle {rel32:.2e}, vs FP64 oracle {rel64:.2e}, "
          f"fp32 vs FP64 oracle {rel_o:.2e}")
    assert rel32 < 1e-4, rel32
    assert rel64 < 1e-2 and rel64 <= 1.5 * rel_o + 1e-4, (rel64, rel_o)
    # deep paths exist: the gradient differs from a 6-bounce frame's
    g6 = gpu_adjoint(scene, settings(16, depth=6, rr_start=3), w)
    assert rel_difference(g6, g_gpu) > 1e-4


def _fd_renderer(scene, st):
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene)
    r.SetCamera(scene.camera)
    r.Resize((scene.width, scene.height))
    r.SetSettings(st)
    return r


def _fd(r, scene, w, m, field, c, h):
    def loss(mats):
        r.UpdateMaterials(mats)
        r.RenderFrame()
        img = r.ColorBuffer().reshape(-1, 4).astype(np.float64)
        return float((img[:, :3] * w[:, :3]).sum())

    # material values are stored as fp16 on upload: step to fp16 values and divide by the step
    # that remains
    mp, mm = scene.materials.copy(), scene.materials.copy()
    if c is None:
        p0 = float(mp[m][field])
        mp[m][field] = np.float32(np.float16(p0 + h))
        mm[m][field] = np.float32(np.float16(p0 - h))
        step = float(mp[m][field]) - float(mm[m][field])
    else:
        p0 = float(mp[m][field][c])
        mp[m][field][c] = np.float32(np.float16(p0 + h))
        mm[m][field][c] = np.float32(np.float16(p0 - h))
        step = float(mp[m][field][c]) - float(mm[m][field][c])
    return (loss(mp) - loss(mm)) / step


def test_gpu_adjoint_matches_finite_differences():
    """Parameters whose change leaves every sampled path unchanged (Lambertian base colours, the
    base colour of a metallic = 1 conductor, emission): central differences of GPU renders with
    common random numbers must agree with the adjoint to 1e-2."""
    scene = tr.cornell_box(width=48, height=48, max_depth=6)
    m = scene.materials.copy()
    for f in ("diffuse", "emissive", "metallic", "roughness", "specular"):
        m[f] = m[f].astype(np.float16).astype(np.float32)
    scene.materials = m
    st = settings(8)
    rng = np.random.default_rng(2)
    w = rng.uniform(-1, 1, (48 * 48, 4)).astype(np.float32)
    w[:, 3] = 0
    g = gpu_adjoint(scene, st, w)
    r = _fd_renderer(scene, st)
    light = int(np.where(scene.materials["emissive"].sum(1) > 0)[0][0])
    checks = [(mi, "diffuse", c, c, 2.0 ** -7) for mi in range(7) for c in range(3)]
    checks += [(light, "emissive", c, 6 + c, 2.0 ** -3) for c in range(3)]
    bad = []
    for mi, field, c, slot, h in checks:
        fd = _fd(r, scene, w, mi, field, c, h)
        if abs(fd - g[mi, slot]) > 1e-2 * abs(fd) + 1e-4:
            bad.append((mi, field, c, fd, float(g[mi, slot])))
    r.close()
    assert not bad, bad


@pytest.mark.parametrize("field,slot,materials,h", [("roughness", 3, (0, 2, 6), 2.0 ** -8),
                                                     ("metallic", 4, (0, 2, 3), 2.0 ** -6),
                                                     ("specular", 5, (0, 2, 3), 2.0 ** -6)])
def test_gpu_adjoint_statistically_consistent_with_fd(field, slot, materials, h):
    """Roughness, metallic and specular move the sampled directions (the GGX lobe's shape, the
    lobe-selection weights) and so rays across geometric edges: the fixed-seed finite difference
    is a noisy estimator of the derivative while the detached-sampling adjoint is not. Over
    independent seeds (batch means) the two must agree within three standard errors of their
    difference; and at least one of them must be resolved (adjoint mean above three standard
    errors), so that a wrong gradient would show. Metallic and specular are checked on walls whose
    values lie inside [h, 1 - h] (metallic 0.12-0.27, specular 0.23-0.80)."""
    scene = diff_scene(256, 256)
    rng = np.random.default_rng(4)
    w = rng.uniform(0.0, 1.0, (256 * 256, 4)).astype(np.float32)
    w[:, 3] = 0
    rows = []
    for mi in materials:
        p0 = float(scene.materials[mi][field])
        assert h <= p0 <= 1.0 - h or field == "roughness"
        diffs = []
        for seed in range(16):
            st = settings(16)
            st.seed = 1000 + seed
            g = gpu_adjoint(scene, st, w)
            r = _fd_renderer(scene, st)
            fd = _fd(r, scene, w, mi, field, None, h)
            r.close()
            diffs.append((fd, float(g[mi, slot])))
        d = np.array(diffs)
        delta = d[:, 0] - d[:, 1]
        se = delta.std(ddof=1) / np.sqrt(len(delta))
        rows.append((mi, d[:, 0].mean(), d[:, 1].mean(), delta.mean(), se))
    print(f"{field} gradient (material, fd mean, adjoint mean, mean difference, standard error):", rows)
    for mi, fdm, adm, dm, se in rows:
        assert abs(dm) <= 3.0 * se + 1e-3 * abs(adm), rows
    assert any(abs(adm) > 3.0 * se for _, _, adm, _, se in rows), "no material with a resolved gradient"


def test_differentiation_configuration():
    """The differentiation configuration: the closed box (diffuse walls and short box, GGX
    conductor) at 512 x 512, 32 spp, 6 bounces, no Russian roulette; L2 loss
    0.5 |img - target|^2 against a target rendered with every Disney parameter + N(0, 0.05)
    (clipped to [0, 1]). Every parameter whose change leaves the sampled paths fixed (the base
    colours of the diffuse materials and of the metallic conductor, the light's emission) is
    checked against central differences of GPU renders with common random numbers, h = 1e-3
    relative to max(1, |p|), divided by the change that remains after the fp16 rounding of
    material values on upload; within 1e-2. The whole gradient table against the FP64 oracle's."""
    W = H = 512
    scene = tr.cornell_box(width=W, height=H, max_depth=6)
    m = scene.materials.copy()
    for f in ("diffuse", "emissive", "metallic", "roughness", "specular"):
        m[f] = m[f].astype(np.float16).astype(np.float32)
    scene.materials = m
    st = settings(32)
    r = _fd_renderer(scene, st)
    r.UpdateMaterials(tr.perturbed_materials(m))
    r.SetSettings(KernelSettings(**{**st.__dict__, "seed": 7}))
    r.RenderFrame()
    target = r.ColorBuffer().reshape(-1, 4).astype(np.float64)
    r.UpdateMaterials(m)
    r.SetSettings(st)
    r.RenderFrame()
    img = r.ColorBuffer().reshape(-1, 4).astype(np.float64)
    w = (img - target).astype(np.float32)
    w[:, 3] = 0
    g = gpu_adjoint(scene, st, w)

    def loss(mats):
        r.UpdateMaterials(mats)
        r.RenderFrame()
        x = r.ColorBuffer().reshape(-1, 4).astype(np.float64)
        return 0.5 * float(((x[:, :3] - target[:, :3]) ** 2).sum())

    light = int(np.where(m["emissive"].sum(1) > 0)[0][0])
    checks = [(mi, "diffuse", c, c) for mi in range(7) for c in range(3)]
    checks += [(light, "emissive", c, 6 + c) for c in range(3)]
    rows, bad = [], []
    gmax = np.abs(g).max()
    for mi, field, c, slot in checks:
        p0 = float(m[mi][field][c])
        h = 1e-3 * max(1.0, abs(p0))
        mp, mm = m.copy(), m.copy()
        mp[mi][field][c] = np.float32(np.float16(p0 + h))
        mm[mi][field][c] = np.float32(np.float16(p0 - h))
        step = float(mp[mi][field][c]) - float(mm[mi][field][c])
        assert step > 0
        fd = (loss(mp) - loss(mm)) / step
        rows.append((mi, field, c, fd, float(g[mi, slot])))
        if abs(fd - g[mi, slot]) > 1e-2 * abs(fd) + 1e-5 * gmax:
            bad.append(rows[-1])
    r.close()
    print("differentiation configuration (material, field, channel, fd, adjoint):", rows)
    assert not bad, bad
    g64 = Oracle(scene).adjoint(scene.camera, st, W, H, 0, w, scale=1.0 / st.multiSample, use_double=True)
    rel = rel_difference(g, g64)
    print(f"differentiation configuration: GPU vs FP64 oracle gradient {rel:.2e}")
    assert rel < 1e-4, rel


def test_torch_autograd_function():
    from trayracer_gb300.autograd import DifferentiableRenderer

    scene = diff_scene(32, 24)
    dr = DifferentiableRenderer(scene, spp=8, max_depth=6, seed=3)
    params = dr.initial_params().cuda().requires_grad_(True)
    img = dr.render(params)
    assert img.shape == (24, 32, 4) and torch.isfinite(img).all()
    target = img.detach() * 0.9
    loss = ((img[..., :3] - target[..., :3]) ** 2).sum()
    loss.backward()
    g = params.grad.detach().cpu().numpy()
    assert np.isfinite(g).all() and np.abs(g).sum() > 0
    # same numbers as the C entry point on the same pixel gradient
    w = (2 * (img - target)).detach().cpu().numpy().reshape(-1, 4).astype(np.float32)
    w[:, 3] = 0
    dr.close()
    g2 = gpu_adjoint(scene, settings(8), w)
    np.testing.assert_allclose(g, g2, rtol=1e-3, atol=1e-5)


def test_adjoint_cost_relative_to_forward():
    scene = diff_scene(256, 256)
    st = settings(32)
    r = tr.DeviceRenderer(0)
    r.UpdateScene(scene)
    r.SetCamera(scene.camera)
    r.Resize((256, 256))
    r.SetSettings(st)
    pg = torch.ones((256, 256, 4), dtype=torch.float32, device="cuda")
    grad = torch.zeros((scene.materials.shape[0], 9), dtype=torch.float32, device="cuda")
    for _ in range(2):
        r.RenderFrame(use_graph=True)
        r.AdjointFrame(pg.data_ptr(), 1.0 / 32, grad.data_ptr())
    torch.cuda.synchronize()
    a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    a.record()
    r.RenderFrame(use_graph=True)
    b.record()
    r.AdjointFrame(pg.data_ptr(), 1.0 / 32, grad.data_ptr())
    c.record()
    torch.cuda.synchronize()
    fwd, adj = a.elapsed_time(b), b.elapsed_time(c)
    print(f"forward {fwd:.3f} ms, adjoint {adj:.3f} ms, ratio {adj / fwd:.2f}")
    r.close()
    assert adj / fwd < 3.0, f"adjoint {adj:.3f} ms vs forward {fwd:.3f} ms"

