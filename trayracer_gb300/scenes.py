"""Seeded procedural scenes for the benchmark configurations.

The reference's own scenes (Resources/scenes/*.json) point at model files of a
submodule that is not part of the reference tree, so these synthetic scenes
stand in for them. Only +, -, *, / and sqrt are used so the arrays are
bit-identical on every platform numpy runs on.
"""
from __future__ import annotations

import dataclasses
import hashlib
from dataclasses import dataclass, field

import numpy as np

from ._abi import TR_CLOSURE_DIFFUSE, TR_CLOSURE_DISNEY, TR_CLOSURE_LAMBERT

MATERIAL_DTYPE = np.dtype(
    [
        ("diffuse", "<f4", (3,)),
        ("emissive", "<f4", (3,)),
        ("metallic", "<f4"),
        ("subsurface", "<f4"),
        ("specular", "<f4"),
        ("roughness", "<f4"),
        ("specular_tint", "<f4"),
        ("anisotropic", "<f4"),
        ("sheen", "<f4"),
        ("sheen_tint", "<f4"),
        ("clearcoat", "<f4"),
        ("clearcoat_gloss", "<f4"),
        ("closure", "<u4"),
    ]
)
assert MATERIAL_DTYPE.itemsize == 68


def material(diffuse=(1.0, 1.0, 1.0), emissive=(0.0, 0.0, 0.0), closure=TR_CLOSURE_DIFFUSE, metallic=0.0,
             subsurface=0.0, specular=0.0, roughness=1.0, specular_tint=0.0, anisotropic=0.0, sheen=0.0,
             sheen_tint=0.0, clearcoat=0.0, clearcoat_gloss=0.0):
    """One material record; defaults follow Material::Material (Tracer/Resources/Material.cpp:102-114)."""
    m = np.zeros((), MATERIAL_DTYPE)
    m["diffuse"] = diffuse
    m["emissive"] = emissive
    m["metallic"] = metallic
    m["subsurface"] = subsurface
    m["specular"] = specular
    m["roughness"] = roughness
    m["specular_tint"] = specular_tint
    m["anisotropic"] = anisotropic
    m["sheen"] = sheen
    m["sheen_tint"] = sheen_tint
    m["clearcoat"] = clearcoat
    m["clearcoat_gloss"] = clearcoat_gloss
    m["closure"] = closure
    return m


@dataclass
class CameraSpec:
    """CameraNode (Tracer/Resources/CameraNode.h): position, target, up, fov in radians."""

    position: tuple = (0.0, 0.0, -1.0)
    target: tuple = (0.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    fov: float = float(np.float32(90.0 * np.pi / 180.0))
    aperture: float = 0.0
    distortion: float = 0.0
    focal_dist: float = 1e5
    bokeh_side_count: int = 0
    bokeh_rotation: float = 0.0

    def basis(self):
        """CameraNode::Transform (Tracer/Resources/CameraNode.cpp:49-63): side, up, forward."""
        f32 = np.float32

        def nrm(v):
            return (v * (f32(1.0) / np.sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))).astype(np.float32)

        pos = np.asarray(self.position, np.float32)
        tgt = np.asarray(self.target, np.float32)
        up = np.asarray(self.up, np.float32)
        fwd = nrm(tgt - pos)
        side = nrm(np.cross(fwd, up).astype(np.float32))
        up2 = nrm(np.cross(side, fwd).astype(np.float32))
        return side, up2, fwd


@dataclass
class Scene:
    name: str
    positions: np.ndarray            # (V, 3) float32
    normals: np.ndarray | None       # (V, 3) float32
    texcoords: np.ndarray | None     # (V, 2) float32
    indices: np.ndarray              # (T, 3) uint32
    material_indices: np.ndarray     # (T,) uint32
    materials: np.ndarray            # (M,) MATERIAL_DTYPE
    camera: CameraSpec = field(default_factory=CameraSpec)
    width: int = 256
    height: int = 256
    spp: int = 16
    max_depth: int = 5
    rr_start: int = 1 << 30
    seed: int = 1
    # textures: (H, W, 4) float16 RGBA arrays; material_textures: (M, 13) texture index per
    # MaterialPropertyIds slot (0xFFFFFFFF: none), or None
    textures: list = field(default_factory=list)
    material_textures: np.ndarray | None = None

    @property
    def triangle_count(self) -> int:
        return int(self.indices.shape[0])

    def digest(self) -> str:
        h = hashlib.sha256()
        for a in (self.positions, self.normals, self.texcoords, self.indices, self.material_indices, self.materials):
            if a is not None:
                h.update(np.ascontiguousarray(a).tobytes())
        if self.material_textures is not None:
            h.update(np.ascontiguousarray(self.material_textures, np.uint32).tobytes())
            for t in self.textures:
                h.update(np.ascontiguousarray(t, np.float16).tobytes())
        return h.hexdigest()[:16]


@dataclass
class InstancedScene(Scene):
    """A two-level scene: meshes (dicts of positions, normals, texcoords, indices, material_indices),
    a material offset per mesh (the reference's MaterialOffsets) and instances (mesh index, 3x4
    object-to-world rows (r | t)). The one-mesh fields hold mesh 0."""

    meshes: list = field(default_factory=list)
    mesh_material_offsets: np.ndarray | None = None
    instances: list = field(default_factory=list)

    @property
    def triangle_count(self) -> int:
        return int(sum(m["indices"].shape[0] for m in self.meshes))

    def digest(self) -> str:
        h = hashlib.sha256(super().digest().encode())
        for m in self.meshes:
            for k in ("positions", "normals", "texcoords", "indices", "material_indices"):
                if m.get(k) is not None:
                    h.update(np.ascontiguousarray(m[k]).tobytes())
        h.update(np.ascontiguousarray(self.mesh_material_offsets, np.uint32).tobytes())
        for mi, xf in self.instances:
            h.update(np.uint32(mi).tobytes())
            h.update(np.asarray(xf, np.float32).tobytes())
        return h.hexdigest()[:16]


def placement(cos_y: float = 1.0, sin_y: float = 0.0, scale: float = 1.0, translate=(0.0, 0.0, 0.0)):
    """Rows (r | t) of a rotation about y (cos, sin given), a uniform scale and a translation."""
    c, s_, k = np.float32(cos_y), np.float32(sin_y), np.float32(scale)
    tx, ty, tz = (np.float32(v) for v in translate)
    return np.array([[k * c, 0, k * s_, tx], [0, k, 0, ty], [-k * s_, 0, k * c, tz]], np.float32)


class _Builder:
    def __init__(self):
        self.pos, self.nrm, self.uv, self.idx, self.mat = [], [], [], [], []
        self.count = 0

    def quad(self, corners, normal, mat):
        c = np.asarray(corners, np.float32)
        base = self.count
        self.pos.append(c)
        self.nrm.append(np.tile(np.asarray(normal, np.float32), (4, 1)))
        self.uv.append(np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32))
        self.idx.append(np.array([[base, base + 1, base + 2], [base, base + 2, base + 3]], np.uint32))
        self.mat.append(np.array([mat, mat], np.uint32))
        self.count += 4

    def box(self, center, size, angle_cos, angle_sin, mat):
        """Axis box rotated about y (cos, sin given exactly)."""
        cx, cy, cz = center
        hx, hy, hz = (s * 0.5 for s in size)
        c, s = np.float32(angle_cos), np.float32(angle_sin)

        def p(x, y, z):
            return (cx + c * x + s * z, cy + y, cz - s * x + c * z)

        def n(x, y, z):
            return (c * x + s * z, y, -s * x + c * z)

        faces = [
            ([p(-hx, -hy, -hz), p(hx, -hy, -hz), p(hx, hy, -hz), p(-hx, hy, -hz)], n(0, 0, -1)),
            ([p(hx, -hy, hz), p(-hx, -hy, hz), p(-hx, hy, hz), p(hx, hy, hz)], n(0, 0, 1)),
            ([p(-hx, -hy, hz), p(-hx, -hy, -hz), p(-hx, hy, -hz), p(-hx, hy, hz)], n(-1, 0, 0)),
            ([p(hx, -hy, -hz), p(hx, -hy, hz), p(hx, hy, hz), p(hx, hy, -hz)], n(1, 0, 0)),
            ([p(-hx, hy, -hz), p(hx, hy, -hz), p(hx, hy, hz), p(-hx, hy, hz)], n(0, 1, 0)),
            ([p(-hx, -hy, hz), p(hx, -hy, hz), p(hx, -hy, -hz), p(-hx, -hy, -hz)], n(0, -1, 0)),
        ]
        for corners, normal in faces:
            self.quad(corners, normal, mat)

    def arrays(self):
        return (np.concatenate(self.pos).astype(np.float32), np.concatenate(self.nrm).astype(np.float32),
                np.concatenate(self.uv).astype(np.float32), np.concatenate(self.idx).astype(np.uint32),
                np.concatenate(self.mat).astype(np.uint32))


def cornell_box(seed: int = 1, width: int = 256, height: int = 256, spp: int = 16, max_depth: int = 5,
                wall_closure: int = TR_CLOSURE_DIFFUSE) -> Scene:
    """Closed box: 5 axis-aligned quad walls (10 tris), 2 rotated boxes (24 tris), 1 quad light (2 tris,
    radiance 15). Walls Lambertian with albedo U[0.2, 0.8]^3, the tall box a GGX conductor (Disney,
    metallic 1, roughness 0.3), the short box Lambertian. Camera: the reference's default camera
    (Apps/Demo/App.cpp:27), at (0, 0, -1) looking at the origin, fov 90 degrees. With
    wall_closure = TR_CLOSURE_LAMBERT every material uses the reference's live Lambert closure."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    mats = []
    walls = [
        ([(-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1)], (0, 1, 0)),   # floor
        ([(-1, 1, 1), (1, 1, 1), (1, 1, -1), (-1, 1, -1)], (0, -1, 0)),     # ceiling
        ([(-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)], (0, 0, -1)),     # back
        ([(-1, -1, -1), (-1, -1, 1), (-1, 1, 1), (-1, 1, -1)], (1, 0, 0)),  # left
        ([(1, -1, 1), (1, -1, -1), (1, 1, -1), (1, 1, 1)], (-1, 0, 0)),     # right
    ]
    for corners, normal in walls:
        albedo = rng.uniform(0.2, 0.8, 3).astype(np.float32)
        mats.append(material(diffuse=albedo, closure=wall_closure))
        b.quad(corners, normal, len(mats) - 1)
    # short Lambertian box, rotated by -0.3 rad about y (cos, sin rounded to float32)
    mats.append(material(diffuse=rng.uniform(0.2, 0.8, 3).astype(np.float32), closure=wall_closure))
    b.box((0.35, -0.7, -0.1), (0.6, 0.6, 0.6), 0.9553365, -0.29552022, len(mats) - 1)
    # tall GGX conductor box, rotated by +0.3 rad
    mats.append(material(diffuse=(0.95, 0.64, 0.54), closure=TR_CLOSURE_DISNEY, metallic=1.0, roughness=0.3,
                         specular=0.5))
    b.box((-0.35, -0.4, 0.35), (0.6, 1.2, 0.6), 0.9553365, 0.29552022, len(mats) - 1)
    # quad area light just below the ceiling, facing down
    mats.append(material(diffuse=(1, 1, 1), emissive=(15, 15, 15), closure=TR_CLOSURE_DIFFUSE))
    b.quad([(-0.25, 0.99, -0.25), (0.25, 0.99, -0.25), (0.25, 0.99, 0.25), (-0.25, 0.99, 0.25)], (0, -1, 0),
           len(mats) - 1)
    pos, nrm, uv, idx, mat = b.arrays()
    mats = np.array(mats, MATERIAL_DTYPE)
    if wall_closure == TR_CLOSURE_LAMBERT:
        # the reference shades every material with its Lambert closure (PathTracing.h:129)
        mats["closure"] = TR_CLOSURE_LAMBERT
    return Scene("cornell_box", pos, nrm, uv, idx, mat, mats, CameraSpec(), width, height, spp, max_depth, 1 << 30,
                 seed)


def perturbed_materials(materials: np.ndarray, seed: int = 2, sigma: float = 0.05) -> np.ndarray:
    """The differentiation target's parameters: every Disney parameter (base colour, roughness,
    metallic, specular) of every non-emissive material + N(0, sigma), clipped to [0, 1]; emitters
    keep theirs."""
    rng = np.random.default_rng(seed)
    m = np.array(materials, MATERIAL_DTYPE, copy=True)
    for key in ("diffuse", "roughness", "metallic", "specular"):
        v = m[key].astype(np.float64) + rng.normal(0.0, sigma, m[key].shape)
        m[key] = np.clip(v, 0.0, 1.0).astype(np.float32)
    emissive = np.asarray(materials["emissive"]).max(axis=-1) > 0
    m[emissive] = np.asarray(materials)[emissive]
    return m


def textured_cornell(seed: int = 5, width: int = 48, height: int = 48, spp: int = 4, max_depth: int = 5,
                     wall_closure: int = TR_CLOSURE_DIFFUSE, tex_size: int = 16) -> Scene:
    """The Cornell box with textures: texture coordinates are a planar projection of the vertex
    positions (ranging beyond [0, 1], so the wrap addressing matters); the walls and the short box
    carry a random diffuse texture, the floor also a roughness, metallic and a normal map whose
    blue channel falls below one half on some texels (the reference applies normal maps before
    its tangent frame exists, so such texels flip the normal), and the light's diffuse is
    textured too (its emission is Emissive times the textured diffuse)."""
    sc = cornell_box(seed=seed, width=width, height=height, spp=spp, max_depth=max_depth, wall_closure=wall_closure)
    rng = np.random.default_rng(seed + 100)
    p = sc.positions
    sc.texcoords = np.stack([p[:, 0] * np.float32(0.73) + p[:, 2] * np.float32(0.41) + np.float32(0.2),
                             p[:, 1] * np.float32(0.67) - p[:, 2] * np.float32(0.29) + np.float32(0.1)],
                            axis=-1).astype(np.float32)

    def tex(lo, hi, shape=(tex_size, tex_size)):
        t = rng.uniform(lo, hi, shape + (4,)).astype(np.float16)
        t[..., 3] = np.float16(1.0)
        return t

    normal = tex(0.0, 1.0)
    normal[..., 2] = np.where(rng.random((tex_size, tex_size)) < 0.2, np.float16(0.3), np.float16(0.9))
    sc.textures = [tex(0.2, 1.0), tex(0.3, 1.0, (8, 12)), tex(0.0, 1.0, (5, 7)), normal]
    mt = np.full((sc.materials.shape[0], 13), 0xFFFFFFFF, np.uint32)
    diffuse, roughness, metallic, nrm = 3, 7, 5, 6
    for m in range(sc.materials.shape[0]):
        if m != 6:  # not the tall conductor box
            mt[m, diffuse] = 0
    mt[0, roughness] = 1   # floor
    mt[0, metallic] = 2
    mt[0, nrm] = 3
    mt[5, nrm] = 3         # short box
    sc.material_textures = mt
    sc.name = "textured_cornell"
    return sc


def instanced_cornell(seed: int = 3, width: int = 64, height: int = 48, spp: int = 4, max_depth: int = 5,
                      wall_closure: int = TR_CLOSURE_DIFFUSE) -> InstancedScene:
    """A two-level Cornell box: the room (5 quads, identity instance), two unit-box meshes placed
    three times (rotated about y, scaled, translated), a sphere mesh placed twice and a quad light
    mesh placed twice (translations only: the reference places light triangles with the transpose
    of the instance rotation, Scene.cpp:288-291, which agrees with the geometry only then)."""
    rng = np.random.default_rng(seed)
    mats = []
    meshes = []
    offsets = []

    def mesh_from(builder, local_mats):
        pos, nrm, uv, idx, mat = builder.arrays()
        offsets.append(len(mats))
        mats.extend(local_mats)
        meshes.append(dict(positions=pos, normals=nrm, texcoords=uv, indices=idx, material_indices=mat))

    room = _Builder()
    walls = [
        ([(-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1)], (0, 1, 0)),
        ([(-1, 1, 1), (1, 1, 1), (1, 1, -1), (-1, 1, -1)], (0, -1, 0)),
        ([(-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)], (0, 0, -1)),
        ([(-1, -1, -1), (-1, -1, 1), (-1, 1, 1), (-1, 1, -1)], (1, 0, 0)),
        ([(1, -1, 1), (1, -1, -1), (1, 1, -1), (1, 1, 1)], (-1, 0, 0)),
    ]
    wall_mats = []
    for k, (corners, normal) in enumerate(walls):
        wall_mats.append(material(diffuse=rng.uniform(0.2, 0.8, 3).astype(np.float32), closure=wall_closure))
        room.quad(corners, normal, k)
    mesh_from(room, wall_mats)
    for closure, kw in ((wall_closure, dict(diffuse=rng.uniform(0.2, 0.8, 3).astype(np.float32))),
                        (TR_CLOSURE_DISNEY, dict(diffuse=(0.95, 0.64, 0.54), metallic=1.0, roughness=0.3,
                                                 specular=0.5))):
        box = _Builder()
        box.box((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 1.0, 0.0, 0)
        mesh_from(box, [material(closure=closure, **kw)])
    sp_p, sp_i = _octahedron_sphere(6)
    mat_s = material(diffuse=rng.uniform(0.3, 0.9, 3).astype(np.float32), closure=TR_CLOSURE_DISNEY,
                     roughness=0.5, metallic=0.2, specular=0.5)
    mats_before = len(mats)
    offsets.append(mats_before)
    mats.append(mat_s)
    meshes.append(dict(positions=sp_p, normals=sp_p.copy(), texcoords=None, indices=sp_i,
                       material_indices=np.zeros(sp_i.shape[0], np.uint32)))
    light = _Builder()
    light.quad([(-0.12, 0.0, -0.12), (0.12, 0.0, -0.12), (0.12, 0.0, 0.12), (-0.12, 0.0, 0.12)], (0, -1, 0), 0)
    mesh_from(light, [material(diffuse=(1, 1, 1), emissive=(20, 20, 20), closure=TR_CLOSURE_DIFFUSE)])
    instances = [
        (0, placement()),
        (1, placement(0.9553365, -0.29552022, 0.6, (0.35, -0.7, -0.1))),
        (1, placement(0.8775826, 0.47942555, 0.3, (-0.55, -0.85, -0.45))),
        (2, placement(0.9553365, 0.29552022, 0.6, (-0.35, -0.4, 0.35))),
        (3, placement(1.0, 0.0, 0.2, (0.45, -0.25, 0.3))),
        (3, placement(0.0, 1.0, 0.12, (-0.1, -0.88, -0.5))),
        (4, placement(translate=(-0.3, 0.99, 0.0))),
        (4, placement(translate=(0.3, 0.99, 0.1))),
    ]
    mats = np.array(mats, MATERIAL_DTYPE)
    if wall_closure == TR_CLOSURE_LAMBERT:
        mats["closure"] = TR_CLOSURE_LAMBERT
    m0 = meshes[0]
    return InstancedScene("instanced_cornell", m0["positions"], m0["normals"], m0["texcoords"], m0["indices"],
                          m0["material_indices"], mats, CameraSpec(), width, height, spp, max_depth, 1 << 30, seed,
                          meshes=meshes, mesh_material_offsets=np.array(offsets, np.uint32), instances=instances)


def _value_noise(n: int, rng: np.random.Generator, octaves: int = 6, base: int = 4) -> np.ndarray:
    """Sum of octaves of smoothstep-interpolated random lattices, values in about [0, 1]."""
    h = np.zeros((n, n), np.float32)
    amp = np.float32(0.5)
    total = np.float32(0.0)
    for o in range(octaves):
        cells = base << o
        lat = rng.random((cells + 1, cells + 1)).astype(np.float32)
        u = (np.arange(n, dtype=np.float32) * np.float32(cells)) / np.float32(n - 1)
        i0 = np.minimum(u.astype(np.int64), cells - 1)
        f = u - i0.astype(np.float32)
        f = f * f * (np.float32(3.0) - np.float32(2.0) * f)
        a = lat[i0][:, i0]
        b = lat[i0][:, i0 + 1]
        c = lat[i0 + 1][:, i0]
        d = lat[i0 + 1][:, i0 + 1]
        fx = f[None, :]
        fy = f[:, None]
        top = a + (b - a) * fx
        bot = c + (d - c) * fx
        h += amp * (top + (bot - top) * fy)
        total += amp
        amp = amp * np.float32(0.5)
    return (h / total).astype(np.float32)


def heightfield(n: int = 1024, seed: int = 1, width: int = 1920, height: int = 1080, spp: int = 64,
                max_depth: int = 8, rr_start: int = 3, n_lights: int = 64, tiles: int = 16,
                extent: float = 10.0, relief: float = 2.5) -> Scene:
    """Value-noise heightfield of (n-1)^2 * 2 triangles over [-extent, extent]^2, 256 Disney materials
    (baseColor/roughness/metallic/specular U[0,1]) assigned per (n/16)^2 tile, and n_lights emissive
    triangles above it with log-uniform intensity in [1, 1000]."""
    rng = np.random.default_rng(seed)
    f32 = np.float32
    h = _value_noise(n, rng) * f32(relief)
    coord = (np.arange(n, dtype=np.float32) * f32(2.0 * extent)) / f32(n - 1) - f32(extent)
    X, Z = np.meshgrid(coord, coord)
    pos = np.stack([X, h, Z], axis=-1).reshape(-1, 3).astype(np.float32)
    # normals from central differences
    step = f32(2.0 * extent) / f32(n - 1)
    hp = np.pad(h, 1, mode="edge")
    dx = (hp[1:-1, 2:] - hp[1:-1, :-2]) / (f32(2.0) * step)
    dz = (hp[2:, 1:-1] - hp[:-2, 1:-1]) / (f32(2.0) * step)
    nx, ny, nz = -dx, np.ones_like(dx), -dz
    inv = f32(1.0) / np.sqrt((nx * nx + ny * ny) + nz * nz)
    nrm = np.stack([nx * inv, ny * inv, nz * inv], axis=-1).reshape(-1, 3).astype(np.float32)
    uvc = np.arange(n, dtype=np.float32) / f32(n - 1)
    U, V = np.meshgrid(uvc, uvc)
    uv = np.stack([U, V], axis=-1).reshape(-1, 2).astype(np.float32)
    # two triangles per cell
    j, i = np.meshgrid(np.arange(n - 1, dtype=np.uint32), np.arange(n - 1, dtype=np.uint32))
    v00 = (i * n + j).ravel()
    v01 = v00 + 1
    v10 = v00 + n
    v11 = v10 + 1
    idx = np.empty((2 * v00.size, 3), np.uint32)
    idx[0::2] = np.stack([v00, v10, v11], axis=-1)
    idx[1::2] = np.stack([v00, v11, v01], axis=-1)
    tile = (n - 1 + tiles - 1) // tiles
    ti = (i.ravel() // tile).astype(np.uint32)
    tj = (j.ravel() // tile).astype(np.uint32)
    cell_mat = ti * tiles + tj
    mat = np.repeat(cell_mat, 2).astype(np.uint32)
    mats = []
    for _ in range(tiles * tiles):
        p = rng.random(4).astype(np.float32)
        base_color = rng.random(3).astype(np.float32)
        mats.append(material(diffuse=base_color, closure=TR_CLOSURE_DISNEY, roughness=p[0], metallic=p[1],
                             specular=p[2]))
    # emissive triangles, facing down, above the terrain
    top = float(h.max())
    lp, ln, luv, li, lm = [], [], [], [], []
    base = pos.shape[0]
    for k in range(n_lights):
        cx, cz = (rng.random(2).astype(np.float32) * f32(2.0 * extent * 0.9) - f32(extent * 0.9))
        cy = f32(top) + f32(1.0) + rng.random(dtype=np.float32) * f32(2.0)
        s = f32(0.3)
        tri = np.array([[cx - s, cy, cz - s], [cx + s, cy, cz - s], [cx, cy, cz + s]], np.float32)
        intensity = np.float32(10.0 ** (3.0 * rng.random()))
        mats.append(material(diffuse=(1, 1, 1), emissive=(intensity, intensity, intensity),
                             closure=TR_CLOSURE_DIFFUSE))
        lp.append(tri)
        ln.append(np.tile(np.array([0, -1, 0], np.float32), (3, 1)))
        luv.append(np.zeros((3, 2), np.float32))
        li.append(np.array([[base + 3 * k, base + 3 * k + 1, base + 3 * k + 2]], np.uint32))
        lm.append(np.array([len(mats) - 1], np.uint32))
    pos = np.concatenate([pos] + lp).astype(np.float32)
    nrm = np.concatenate([nrm] + ln).astype(np.float32)
    uv = np.concatenate([uv] + luv).astype(np.float32)
    idx = np.concatenate([idx] + li).astype(np.uint32)
    mat = np.concatenate([mat] + lm).astype(np.uint32)
    cam = CameraSpec(position=(0.0, 9.0, -17.0), target=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0),
                     fov=float(np.float32(60.0 * np.pi / 180.0)))
    return Scene(f"heightfield_{n}", pos, nrm, uv, idx, mat, np.array(mats, MATERIAL_DTYPE), cam, width, height,
                 spp, max_depth, rr_start, seed)


def outdoor_heightfield(n: int = 16, width: int = 32, height: int = 24, n_lights: int = 4,
                        lambert: bool = False) -> Scene:
    """The heightfield seen toward its horizon, so that paths leave it and see the sky; with
    lambert=True every material uses the reference's live Lambert closure."""
    sc = heightfield(n=n, width=width, height=height, n_lights=n_lights)
    sc.name = f"outdoor_heightfield_{n}"
    sc.camera = dataclasses.replace(sc.camera, target=(0.0, 4.0, 0.0))
    if lambert:
        sc.materials["closure"] = TR_CLOSURE_LAMBERT
    return sc


def random_soup(n_tris: int = 2000, seed: int = 7, extent: float = 1.0) -> Scene:
    """Random triangles in a cube, for traversal tests."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-extent, extent, (n_tris, 1, 3)).astype(np.float32)
    offs = rng.normal(0, 0.08 * extent, (n_tris, 3, 3)).astype(np.float32)
    pos = (centers + offs).reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * n_tris, dtype=np.uint32).reshape(-1, 3)
    mats = np.array([material(diffuse=(0.5, 0.5, 0.5))], MATERIAL_DTYPE)
    return Scene("soup", pos, None, None, idx, np.zeros(n_tris, np.uint32), mats,
                 CameraSpec(position=(0.0, 0.0, -3.0)), 64, 64, 1, 1)


def _octahedron_sphere(subdiv: int):
    """Unit sphere from an octahedron whose faces are cut into subdiv^2 triangles each (8 subdiv^2
    triangles); grid points are projected onto the sphere with a square root only."""
    f32 = np.float32
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    faces = []
    for sx in (0, 1):
        for sy in (2, 3):
            for sz in (4, 5):
                a, b, c = axes[sx], axes[sy], axes[sz]
                # keep the winding outward
                if float(np.dot(np.cross(b - a, c - a), a + b + c)) < 0.0:
                    b, c = c, b
                faces.append((a, b, c))
    n = subdiv
    ii, jj = [], []
    for i in range(n + 1):
        for j in range(n + 1 - i):
            ii.append(i)
            jj.append(j)
    ii = np.array(ii, np.int64)
    jj = np.array(jj, np.int64)
    lookup = -np.ones((n + 1, n + 1), np.int64)
    lookup[ii, jj] = np.arange(ii.size)
    tri = []
    for i in range(n):
        for j in range(n - i):
            tri.append((lookup[i, j], lookup[i + 1, j], lookup[i, j + 1]))
            if i + j < n - 1:
                tri.append((lookup[i + 1, j], lookup[i + 1, j + 1], lookup[i, j + 1]))
    tri = np.array(tri, np.int64)
    pos, idx = [], []
    for a, b, c in faces:
        wa = (f32(n) - ii - jj).astype(np.float32)[:, None]
        p = (wa * a + ii.astype(np.float32)[:, None] * b + jj.astype(np.float32)[:, None] * c) / f32(n)
        inv = f32(1.0) / np.sqrt((p[:, 0] * p[:, 0] + p[:, 1] * p[:, 1]) + p[:, 2] * p[:, 2])
        idx.append(tri + len(pos) * ii.size)
        pos.append((p * inv[:, None]).astype(np.float32))
    return np.concatenate(pos).astype(np.float32), np.concatenate(idx).astype(np.uint32)


def sphere_scene(seed: int, triangles: int, width: int, height: int, spp: int, n_lights: int,
                 max_depth: int = 6) -> Scene:
    """Tessellated spheres (radius U[0.1, 2]) in a 20^3 box over a floor, about `triangles`
    triangles in total, lit by n_lights downward emissive triangles (log-uniform intensity in
    [10, 1000]); 4 Disney materials."""
    rng = np.random.default_rng(seed)
    f32 = np.float32
    subdiv = 2
    while 8 * (2 * subdiv) ** 2 <= triangles // 2 and subdiv < 128:
        subdiv *= 2
    per = 8 * subdiv * subdiv
    count = max(1, int(round(triangles / per)))
    unit_p, unit_i = _octahedron_sphere(subdiv)
    mats = []
    for _ in range(4):
        p = rng.random(3).astype(np.float32)
        mats.append(material(diffuse=rng.random(3).astype(np.float32) * f32(0.8) + f32(0.1),
                             closure=TR_CLOSURE_DISNEY, roughness=f32(0.2) + f32(0.8) * p[0], metallic=p[1],
                             specular=p[2]))
    pos, nrm, idx, mat = [], [], [], []
    base = 0
    for _ in range(count):
        c = rng.uniform(-8.0, 8.0, 3).astype(np.float32)
        r = f32(0.1) + f32(1.9) * rng.random(dtype=np.float32)
        pos.append((unit_p * r + c).astype(np.float32))
        nrm.append(unit_p)
        idx.append(unit_i + np.uint32(base))
        mat.append(np.full(unit_i.shape[0], rng.integers(0, 4), np.uint32))
        base += unit_p.shape[0]
    # floor
    fl = np.array([[-10, -10, -10], [10, -10, -10], [10, -10, 10], [-10, -10, 10]], np.float32)
    pos.append(fl)
    nrm.append(np.tile(np.array([0, 1, 0], np.float32), (4, 1)))
    idx.append(np.array([[base, base + 2, base + 1], [base, base + 3, base + 2]], np.uint32))
    mat.append(np.zeros(2, np.uint32))
    base += 4
    for k in range(n_lights):
        cx, cz = rng.uniform(-8.0, 8.0, 2).astype(np.float32)
        cy = f32(10.0)
        s = f32(0.8)
        pos.append(np.array([[cx - s, cy, cz - s], [cx + s, cy, cz - s], [cx, cy, cz + s]], np.float32))
        nrm.append(np.tile(np.array([0, -1, 0], np.float32), (3, 1)))
        intensity = np.float32(10.0 * 100.0 ** rng.random())
        mats.append(material(diffuse=(1, 1, 1), emissive=(intensity, intensity, intensity),
                             closure=TR_CLOSURE_DIFFUSE))
        idx.append(np.array([[base, base + 1, base + 2]], np.uint32))
        mat.append(np.array([len(mats) - 1], np.uint32))
        base += 3
    cam = CameraSpec(position=(0.0, 4.0, -28.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                     fov=float(np.float32(60.0 * np.pi / 180.0)))
    return Scene(f"spheres_{seed}", np.concatenate(pos).astype(np.float32), np.concatenate(nrm).astype(np.float32),
                 None, np.concatenate(idx).astype(np.uint32), np.concatenate(mat).astype(np.uint32),
                 np.array(mats, MATERIAL_DTYPE), cam, width, height, spp, max_depth, 1 << 30, seed)


def sphere_batch(count: int = 64, seed: int = 11, min_tris: int = 1000, max_tris: int = 500_000,
                 resolutions=(128, 256, 512, 1024), spps=(4, 16, 64)) -> list[Scene]:
    """The batching mix: `count` independent seeded scenes with triangle counts log-uniform in
    [min_tris, max_tris], square resolutions and spp drawn uniformly from the given sets, 1-16
    emissive triangles each, 6 bounces."""
    rng = np.random.default_rng(seed)
    ratio = max_tris / min_tris
    out = []
    for k in range(count):
        tris = int(round(min_tris * ratio ** float(rng.random())))
        res = int(resolutions[rng.integers(0, len(resolutions))])
        spp = int(spps[rng.integers(0, len(spps))])
        lights = int(rng.integers(1, 17))
        out.append(sphere_scene(seed * 1000 + k, tris, res, res, spp, lights))
    return out


def displaced_spheres(count: int = 4096, subdiv: int = 25, n_emissive: int = 20, seed: int = 13,
                      width: int = 3840, height: int = 2160, spp: int = 16, max_depth: int = 12, rr_start: int = 3,
                      extent: float = 40.0) -> Scene:
    """The large configuration: `count` spheres of 8 subdiv^2 triangles (25 -> 5000, 4096 spheres ->
    20.48 M triangles) with every vertex displaced along its normal by N(0, 0.02) of the radius,
    one Disney material per sphere (baseColor/roughness/metallic/specular U[0,1]), and the
    triangles of `n_emissive` spheres emissive (20 x 5000 = 100k emissive triangles) with
    log-uniform intensity in [1, 1000] per sphere."""
    rng = np.random.default_rng(seed)
    f32 = np.float32
    unit_p, unit_i = _octahedron_sphere(subdiv)
    nv, nt = unit_p.shape[0], unit_i.shape[0]
    centers = rng.uniform(-extent, extent, (count, 1, 3)).astype(np.float32)
    radii = (f32(0.5) + f32(1.5) * rng.random((count, 1, 1), dtype=np.float32)).astype(np.float32)
    disp = (f32(1.0) + f32(0.02) * rng.standard_normal((count, nv, 1)).astype(np.float32)).astype(np.float32)
    pos = (centers + unit_p[None, :, :] * (radii * disp)).reshape(-1, 3).astype(np.float32)
    nrm = np.broadcast_to(unit_p[None], (count, nv, 3)).reshape(-1, 3).astype(np.float32)
    idx = (unit_i[None, :, :].astype(np.uint64) + (np.arange(count, dtype=np.uint64) * nv)[:, None, None])
    idx = idx.reshape(-1, 3).astype(np.uint32)
    mat = np.repeat(np.arange(count, dtype=np.uint32), nt)
    emissive = set(int(x) for x in rng.choice(count, size=n_emissive, replace=False))
    mats = []
    for k in range(count):
        p = rng.random(4).astype(np.float32)
        base = rng.random(3).astype(np.float32)
        if k in emissive:
            intensity = np.float32(10.0 ** (3.0 * p[3]))
            mats.append(material(diffuse=(1, 1, 1), emissive=(intensity, intensity, intensity),
                                 closure=TR_CLOSURE_DIFFUSE))
        else:
            mats.append(material(diffuse=base, closure=TR_CLOSURE_DISNEY, roughness=p[0], metallic=p[1],
                                 specular=p[2]))
    cam = CameraSpec(position=(0.0, 10.0, -extent * 2.2), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                     fov=float(np.float32(60.0 * np.pi / 180.0)))
    return Scene(f"displaced_spheres_{count}", pos, nrm, None, idx, mat, np.array(mats, MATERIAL_DTYPE), cam,
                 width, height, spp, max_depth, rr_start, seed)


CONFIGS = {
    "cornell_box": cornell_box,
    "heightfield": heightfield,
    "sphere_batch": sphere_batch,
    "displaced_spheres": displaced_spheres,
}
