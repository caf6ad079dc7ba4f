"""The GPU path-replay adjoint: against the FP64 oracle's gradient of the same
estimator, against central finite differences of GPU renders (parameters
whose change leaves the sampled paths fixed), and through the libtorch
autograd function. Firefly clamp off (its scale is not differentiated)."""
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


def settings(spp, depth=6):
    return KernelSettings(multiSample=spp, maxDepth=depth, seed=3, rrStart=1 << 30, maxColor=1e30)


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
    big = np.abs(g_cpu) > 1e-2 * np.abs(g_cpu).max()
    rel = np.linalg.norm(g_gpu[big] - g_cpu[big]) / np.linalg.norm(g_cpu[big])
    print(f"relative gradient difference GPU vs FP64 oracle: {rel:.2e}")
    assert rel < 2e-2, rel


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

    mp, mm = scene.materials.copy(), scene.materials.copy()
    if c is None:
        mp[m][field] += h
        mm[m][field] -= h
    else:
        mp[m][field][c] += h
        mm[m][field][c] -= h
    return (loss(mp) - loss(mm)) / (2 * h)


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


def test_gpu_adjoint_roughness_statistically_consistent_with_fd():
    """Roughness moves the sampled GGX directions (and rays across geometric edges), so the
    fixed-seed finite difference is a noisy estimator of the derivative while the
    detached-sampling adjoint is not. Over independent seeds (batch means) the two must agree
    within three standard errors of their difference."""
    scene = diff_scene(128, 128)
    rng = np.random.default_rng(4)
    w = rng.uniform(0.0, 1.0, (128 * 128, 4)).astype(np.float32)
    w[:, 3] = 0
    h = 2.0 ** -8
    rows = []
    for mi in (0, 2, 6):
        diffs = []
        for seed in range(12):
            st = settings(16)
            st.seed = 1000 + seed
            g = gpu_adjoint(scene, st, w)
            r = _fd_renderer(scene, st)
            fd = _fd(r, scene, w, mi, "roughness", None, h)
            r.close()
            diffs.append((fd, float(g[mi, 3])))
        d = np.array(diffs)
        delta = d[:, 0] - d[:, 1]
        se = delta.std(ddof=1) / np.sqrt(len(delta))
        rows.append((mi, d[:, 0].mean(), d[:, 1].mean(), delta.mean(), se))
    print("roughness gradient (material, fd mean, adjoint mean, mean difference, standard error):", rows)
    for mi, fdm, adm, dm, se in rows:
        assert abs(dm) <= 3.0 * se + 1e-3 * abs(adm), rows


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

