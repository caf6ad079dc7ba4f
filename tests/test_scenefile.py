"""Scene files (SceneFile::Load, Tracer/FileIO/SceneFile.cpp) and the model / texture cache formats
(ModelFile.cpp, TextureFile.cpp, BinaryFile.inl) read by the library into a two-level scene. Scenes
are rendered from synthetic scene files; the reference's own scene files, where its sources are
present, are only parsed (the models they name are not present)."""
import json
import struct
from pathlib import Path

import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle
from oracle.build import reference_root
from trayracer_gb300.scenefile import load_scene_file, write_model_cache, write_texture_cache
from trayracer_gb300.scenes import MATERIAL_DTYPE, material

# the reference's own scene files, where its sources are present (oracle.build.reference_root)
_REF = reference_root()
REFERENCE_SCENES = _REF / "Resources" / "scenes" if _REF is not None else Path("/nonexistent")


def _box(lo, hi):
    """An axis-aligned box as 12 triangles (8 vertices)."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    p = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
    f = [(0, 1, 2, 3), (5, 4, 7, 6), (4, 0, 3, 7), (1, 5, 6, 2), (3, 2, 6, 7), (4, 5, 1, 0)]
    idx = np.array([t for a, b, c, d in f for t in ((a, b, c), (a, c, d))], np.uint32)
    return p, idx


def _mats(*specs):
    return np.array([material(**s) for s in specs], MATERIAL_DTYPE)


def _m34(m12):
    """float3x4 from a JSON matrix: basis vectors x, y, z then the translation."""
    m = np.asarray(m12, np.float32)
    return dict(x=m[0:3].copy(), y=m[3:6].copy(), z=m[6:9].copy(), t=m[9:12].copy())


def _mul(a, b):
    """transform(float3x4, float3x4) of LinearMath.h in float32: rows of a against columns of b."""
    f = np.float32
    col = [np.array([b["x"][k], b["y"][k], b["z"][k]], f) for k in range(3)]
    dot = lambda u, v: (u[0] * v[0] + u[1] * v[1]) + u[2] * v[2]  # noqa: E731
    return dict(x=np.array([dot(a["x"], c) for c in col], f), y=np.array([dot(a["y"], c) for c in col], f),
                z=np.array([dot(a["z"], c) for c in col], f),
                t=np.array([dot(a["t"], col[k]) + b["t"][k] for k in range(3)], f))


def _rows(m):
    """OptixInstance::transform: the float3x4 as it lies in memory."""
    return np.concatenate([m["x"], m["t"][0:1], m["y"], m["t"][1:2], m["z"], m["t"][2:3]]).reshape(3, 4)


@pytest.fixture()
def scene_dir(tmp_path):
    room_p, room_i = _box((-2, -2, -2), (2, 2, 2))
    write_model_cache(tmp_path / "room.bin", room_p, room_i, np.repeat(np.arange(2, dtype=np.uint32), 6)[:12],
                      _mats(dict(diffuse=(0.7, 0.7, 0.7)), dict(diffuse=(0.2, 0.5, 0.2))), ["walls", "floor"],
                      texcoords=room_p[:, :2] * 0.25)
    box_p, box_i = _box((-0.3, -0.3, -0.3), (0.3, 0.3, 0.3))
    write_model_cache(tmp_path / "box.bin", box_p, box_i, np.zeros(12, np.uint32),
                      _mats(dict(diffuse=(0.9, 0.1, 0.1))), ["red"],
                      texture_paths=[["", "", "", "", "", "", "", "", "", "", "", "", ""]])
    rng = np.random.default_rng(4)
    tex = rng.uniform(0.2, 1.0, (4, 6, 4)).astype(np.float16)
    write_texture_cache(tmp_path / "wall_diffuse.bin", tex)
    # an OBJ light: one quad with an emissive material from its mtllib
    (tmp_path / "light.mtl").write_text("newmtl lamp\nKd 1 1 1\nKe 8 8 8\n")
    (tmp_path / "light.obj").write_text("mtllib light.mtl\nv -0.5 1.9 -0.5\nv 0.5 1.9 -0.5\nv 0.5 1.9 0.5\n"
                                        "v -0.5 1.9 0.5\nusemtl lamp\nf 1 2 3 4\n")
    doc = {
        "models": [{"name": "room", "path": "room.bin"}, {"name": "box", "path": "box.bin"},
                   {"name": "light", "path": "light.obj"}, {"name": "unused", "path": "nowhere.bin"}],
        "instances": [
            {"name": "room", "model": "room",
             "transform": [{"matrix": [1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0]}]},
            {"name": "box a", "model": "box",
             "transform": [{"translate": [0.5, -1.2, 0.3]}, {"rotate-y": 30.0}, {"scale": 1.5}]},
            {"model": "box", "transform": [{"scale": [1.0, 2.0, 0.5]}, {"rotate-x": -20.0},
                                           {"translate": [-0.8, -1.0, 0.6]}]},
            {"name": "lamp", "model": "light"},
            {"name": "ghost", "model": "undeclared"},
        ],
        "materials": [
            {"model": "room", "materials": [
                {"name": "walls", "diffuse": [0.6, 0.6, 0.55], "roughness": 0.4, "diffuseMap": "wall_diffuse.bin"},
                {"name": "floor", "diffuse": 0.3, "metallicMap": "missing_texture.bin"},
                {"name": "no such material", "diffuse": [1, 0, 0]}]},
            {"model": "box", "materials": [{"name": "red", "emissive": [0.0, 0.0, 0.0], "specular": 0.5}]},
        ],
        "camera": {"position": [0.0, 0.5, -1.8], "target": [0.0, 0.0, 0.0], "up": [0.0, 2.0, 0.0], "fov": 75.0,
                   "aperture": 0.01, "focaldist": 2.0, "bokehsides": 6, "bokehrotation": 0.5},
        "renderer": {"multisample": 2, "maxdepth": 6, "aodist": 0.5, "zdepthmax": 4.0, "ray-epsilon": 0.002},
        "sky": {"enabled": False, "dir": [0.0, 2.0, 1.0], "turbidity": 5.0, "intensity": 500.0},
        "post": [{"name": "ignored", "frag": "x.frag"}],
    }
    (tmp_path / "scene.json").write_text(json.dumps(doc, indent=2))
    return tmp_path, doc, tex


def test_scene_file_contents(scene_dir):
    d, doc, tex = scene_dir
    sf = load_scene_file("scene.json", base_dir=d)
    sc = sf.scene
    # meshes in first use among the instances; the undeclared model's instance is left out
    assert sf.mesh_names == ["room", "box", "light"]
    assert sf.instance_names == ["room", "box a", "box", "lamp"]
    assert [m for m, _ in sc.instances] == [0, 1, 1, 2]
    np.testing.assert_array_equal(sc.mesh_material_offsets, [0, 2, 3])
    assert sf.material_names == ["walls", "floor", "red", "lamp"]
    # the texture that cannot be read is reported and left out
    assert any("missing_texture.bin" in w for w in sf.warnings), sf.warnings
    # instance transforms: the operations composed as float3x4 products
    ident = _m34([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0])
    np.testing.assert_array_equal(sc.instances[0][1], _rows(ident))
    tr_ = _m34([1, 0, 0, 0, 1, 0, 0, 0, 1, 0.5, -1.2, 0.3])
    a = np.float32(30.0) * (np.float32(3.14159265359) / np.float32(180.0))
    s, c = np.float32(np.sin(a)), np.float32(np.cos(a))
    rot = _m34([c, 0, -s, 0, 1, 0, s, 0, c, 0, 0, 0])
    sca = _m34([1.5, 0, 0, 0, 1.5, 0, 0, 0, 1.5, 0, 0, 0])
    want = _mul(_mul(_mul(ident, tr_), rot), sca)
    np.testing.assert_allclose(sc.instances[1][1], _rows(want), rtol=1e-6, atol=1e-7)
    # materials: JSON overrides on the cached materials; a single number sets the first channel
    m = sc.materials
    np.testing.assert_allclose(m["diffuse"][0], [0.6, 0.6, 0.55], rtol=1e-7)
    assert m["roughness"][0] == np.float32(0.4)
    np.testing.assert_allclose(m["diffuse"][1], [0.3, 0.5, 0.2], rtol=1e-7)
    assert m["specular"][2] == np.float32(0.5)
    np.testing.assert_array_equal(m["emissive"][3], [8, 8, 8])
    assert (m["closure"] == tr.TR_CLOSURE_LAMBERT).all()
    # textures: the walls' diffuse map from the texture cache
    assert len(sc.textures) == 1
    np.testing.assert_array_equal(sc.textures[0], tex)
    assert sc.material_textures[0, 3] == 0 and (sc.material_textures[1:] == 0xFFFFFFFF).all()
    # camera: CameraNode with a normalised up, fov in radians
    cam = sf.camera
    assert cam.up == (0.0, 1.0, 0.0)
    assert cam.fov == pytest.approx(75.0 * 3.14159265359 / 180.0, rel=1e-6)
    assert cam.bokeh_side_count == 6 and cam.focal_dist == 2.0
    # renderer and sky sections over their defaults
    st = sf.settings
    assert (st.multiSample, st.maxDepth, st.aoDist, st.zDepthMax) == (2, 6, 0.5, 4.0)
    assert st.rayEpsilon == np.float32(0.002)
    assert not sf.sky.enabled and sf.sky.drawSun and sf.sky.turbidity == 5.0 and sf.sky.sunIntensity == 500.0


def test_model_cache_round_trip(scene_dir):
    d, _, _ = scene_dir
    raw = (d / "box.bin").read_bytes()
    assert raw[:4] == b"MDL\x02"
    # eight vertices of float3, a 64-bit count first
    assert struct.unpack_from("<Q", raw, 4)[0] == 8
    sf = load_scene_file("scene.json", base_dir=d)
    box_p, box_i = _box((-0.3, -0.3, -0.3), (0.3, 0.3, 0.3))
    mesh = sf.scene.meshes[1]
    np.testing.assert_array_equal(mesh["positions"], box_p)
    np.testing.assert_array_equal(mesh["indices"], box_i)
    np.testing.assert_array_equal(mesh["texcoords"], np.zeros((8, 2), np.float32))
    assert (d / "wall_diffuse.bin").read_bytes()[:4] == b"TEX\x02"


def test_obj_reader(tmp_path):
    (tmp_path / "q.obj").write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
                                    "f 1/1 2/2 3/3 4/4\nf -4/-4 -2/-2 -1/-1\n")
    (tmp_path / "s.json").write_text(json.dumps({"models": [{"name": "q", "path": "q.obj"}],
                                                 "instances": [{"model": "q"}]}))
    sc = load_scene_file("s.json", base_dir=tmp_path).scene
    m = sc.meshes[0]
    # the quad's fan (0 1 2)(0 2 3) and the repeated triangle share vertices
    np.testing.assert_array_equal(m["indices"], [[0, 1, 2], [0, 2, 3], [0, 2, 3]])
    np.testing.assert_array_equal(m["texcoords"], [[0, 0], [1, 0], [1, 1], [0, 1]])
    # missing normals: the face normal (+z)
    np.testing.assert_allclose(m["normals"], np.tile([0, 0, 1], (4, 1)), atol=1e-7)
    # a default material (diffuse 1, roughness 1)
    assert sc.materials["roughness"][0] == 1.0


def test_scene_file_defaults_and_errors(tmp_path):
    (tmp_path / "empty.json").write_text("{}")
    sf = load_scene_file(tmp_path / "empty.json")
    assert sf.scene is None
    assert sf.sky.enabled and sf.sky.sunIntensity == 1000.0 and sf.sky.turbidity == 4.0
    assert sf.settings.maxDepth == 16 and sf.settings.multiSample == 1
    assert sf.camera.position == (0.0, 0.0, -1.0) and sf.camera.fov == pytest.approx(np.pi / 2, rel=1e-6)
    (tmp_path / "bad.json").write_text('{"models": [1, 2,]}')
    with pytest.raises(tr.TracerError, match="valid json"):
        load_scene_file(tmp_path / "bad.json")
    with pytest.raises(tr.TracerError, match="cannot read"):
        load_scene_file(tmp_path / "absent.json")
    (tmp_path / "trunc.bin").write_bytes(b"MDL\x02" + struct.pack("<Q", 10**6))
    (tmp_path / "t.json").write_text(json.dumps({"models": [{"name": "t", "path": "trunc.bin"}],
                                                 "instances": [{"model": "t"}]}))
    sf = load_scene_file("t.json", base_dir=tmp_path)
    assert sf.scene is None and any("truncated" in w for w in sf.warnings)


def test_scene_file_renders_in_the_oracle(scene_dir):
    """The loaded two-level scene is a valid scene: the oracle renders it (the box lit by the OBJ lamp)."""
    d, _, _ = scene_dir
    sf = load_scene_file("scene.json", base_dir=d, width=16, height=12)
    st = tr.settings_for(sf.scene, multi_sample=2)
    acc, _, _ = Oracle(sf.scene).render(sf.camera, st, 16, 12)
    assert np.isfinite(acc).all() and acc[:, :3].mean() > 0


@pytest.mark.skipif(not REFERENCE_SCENES.is_dir(), reason="reference scene files absent")
@pytest.mark.parametrize("name", ["cornell.json", "sponza.json", "toad_on_a_plane.json", "modernroom.json"])
def test_reference_scene_files_parse(name):
    """The reference's own scene files: their models are absent (reported, left out); the camera,
    renderer and sky sections read as the JSON says."""
    path = REFERENCE_SCENES / name
    doc = json.loads(path.read_text())
    sf = load_scene_file(path, base_dir=REFERENCE_SCENES)
    assert sf.scene is None and len(sf.warnings) >= 1
    if "camera" in doc:
        assert sf.camera.position == pytest.approx(tuple(doc["camera"]["position"]), rel=1e-6)
        if "fov" in doc["camera"]:
            fov = min(max(doc["camera"]["fov"], 0.1), 179.9)
            assert sf.camera.fov == pytest.approx(fov * 3.14159265359 / 180.0, rel=1e-6)
    if "renderer" in doc and "maxdepth" in doc["renderer"]:
        assert sf.settings.maxDepth == doc["renderer"]["maxdepth"]
    if "sky" in doc and "enabled" in doc["sky"]:
        assert sf.sky.enabled == doc["sky"]["enabled"]
        if "turbidity" in doc["sky"]:
            assert sf.sky.turbidity == pytest.approx(doc["sky"]["turbidity"], rel=1e-6)


@pytest.mark.gpu
def test_gpu_renders_a_scene_file(scene_dir):
    """A scene file through the device: sky, settings and camera as loaded; every path's radiance
    against the oracle's (default sampling)."""
    d, _, _ = scene_dir
    sf = load_scene_file("scene.json", base_dir=d, width=32, height=24)
    sc = sf.scene
    st = tr.KernelSettings(**{**sf.settings.__dict__, "seed": 3})
    r = tr.DeviceRenderer(0)
    try:
        r.UpdateScene(sc)
        r.SetCamera(sf.camera)
        r.Resize((sc.width, sc.height))
        r.SetSky(sf.sky)
        r.RenderFrame(st)
        buf = r.Buffers()
        rad = r.read_device(buf["radiance"], np.float32, buf["capacity"] * 4).reshape(st.multiSample, -1, 4)
        stats = r.Statistics()
    finally:
        r.close()
    assert stats["device_error"] == 0
    o = Oracle(sc)
    o.set_sky(sf.sky)
    _, paths, _ = o.render(sf.camera, st, sc.width, sc.height, want_paths=True)
    ok = np.isclose(rad[..., :3].astype(np.float64), paths[..., :3], rtol=1e-2, atol=1e-4).all(-1)
    assert ok.mean() >= 0.97, ok.mean()
    assert paths[..., :3].mean() > 0
