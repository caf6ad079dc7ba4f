"""Scene files of the reference renderer (Tracer/FileIO/SceneFile.cpp) through the library's
scene-file reader (tr_scene_file_load): the scene JSON with its models (the reference's model
cache format or Wavefront OBJ) and textures (its texture cache format), plus writers of the two
cache formats (ModelFile.cpp / TextureFile.cpp SaveToCache)."""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .renderer import KernelSettings, SkySettings, TracerError
from .scenes import MATERIAL_DTYPE, CameraSpec, InstancedScene


@dataclass
class SceneFile:
    """What SceneFile::Load hands the renderer: the scene (None when nothing is placed), the
    camera, the render settings (with aoDist / zDepthMax) and the sky, plus the names."""

    scene: InstancedScene | None
    camera: CameraSpec
    settings: KernelSettings
    sky: SkySettings
    mesh_names: list = field(default_factory=list)
    instance_names: list = field(default_factory=list)
    material_names: list = field(default_factory=list)
    warnings: list = field(default_factory=list)   # models / textures that could not be read


def _array(ptr, dtype, count):
    if count == 0 or not ptr:
        return np.zeros(0, dtype)
    ctype = np.ctypeslib.as_ctypes_type(dtype)
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(count,)).copy()


def _check(lib, st, where):
    if st != 0:
        raise TracerError(st, where, lib.tr_scene_file_last_error().decode(errors="replace"))


def load_scene_file(path: str | os.PathLike, base_dir: str | os.PathLike | None = None, width: int = 256,
                    height: int = 256) -> SceneFile:
    """Reads a scene file; relative paths resolve against base_dir (default: the current
    directory, as the reference resolves them)."""
    lib = _abi.load_library()
    h = C.c_void_p()
    _check(lib, lib.tr_scene_file_load(os.fsencode(path), None if base_dir is None else os.fsencode(base_dir),
                                       C.byref(h)), "tr_scene_file_load")
    try:
        info = _abi.SceneFileInfo()
        _check(lib, lib.tr_scene_file_get_info(h, C.byref(info)), "tr_scene_file_get_info")
        names = lambda p, n: [p[i].decode(errors="replace") for i in range(n)]  # noqa: E731
        st = info.settings
        settings = KernelSettings(multiSample=st.multi_sample, maxDepth=st.max_depth, seed=st.seed,
                                  aoDist=info.ao_dist, zDepthMax=info.z_depth_max, rayEpsilon=st.ray_epsilon,
                                  rrStart=st.rr_start, flags=st.flags, maxColor=st.max_color)
        sk = info.sky
        sky = SkySettings(bool(sk.enabled), bool(sk.draw_sun), tuple(sk.sun_dir), sk.sun_angular_diameter,
                          sk.sun_intensity, sk.turbidity, sk.selection_bias)
        cam = info.camera
        camera = CameraSpec(position=tuple(cam.position), target=tuple(info.camera_target),
                            up=tuple(info.camera_up), fov=float(cam.fov), aperture=cam.aperture,
                            distortion=cam.distortion, focal_dist=cam.focal_dist,
                            bokeh_side_count=cam.bokeh_side_count, bokeh_rotation=cam.bokeh_rotation)
        scene = None
        material_names = []
        if info.scene:
            d = info.scene.contents
            material_names = names(info.material_names, d.material_count)
            meshes = []
            for i in range(d.mesh_count):
                m = d.meshes[i]
                nv, nt = m.vertex_count, m.triangle_count
                meshes.append(dict(
                    positions=_array(m.positions, np.float32, 3 * nv).reshape(nv, 3),
                    normals=_array(m.normals, np.float32, 3 * nv).reshape(nv, 3),
                    texcoords=_array(m.texcoords, np.float32, 2 * nv).reshape(nv, 2),
                    indices=_array(m.indices, np.uint32, 3 * nt).reshape(nt, 3),
                    material_indices=_array(m.material_indices, np.uint32, nt)))
            mats = np.frombuffer(C.string_at(C.cast(d.materials, C.c_void_p), d.material_count *
                                             MATERIAL_DTYPE.itemsize), MATERIAL_DTYPE).copy()
            offsets = _array(d.mesh_material_offsets, np.uint32, d.mesh_count)
            instances = [(int(d.instances[i].mesh), np.array(d.instances[i].transform, np.float32).reshape(3, 4))
                         for i in range(d.instance_count)]
            textures, mat_tex = [], None
            if d.texture_count:
                tds = C.cast(d.textures, C.POINTER(_abi.TextureDesc))
                for i in range(d.texture_count):
                    t = tds[i]
                    textures.append(_array(t.texels, np.uint16, 4 * t.width * t.height)
                                    .view(np.float16).reshape(t.height, t.width, 4))
                mat_tex = _array(d.material_textures, np.uint32, 13 * d.material_count).reshape(-1, 13)
            m0 = meshes[0]
            scene = InstancedScene(os.path.basename(os.fspath(path)), m0["positions"], m0["normals"],
                                   m0["texcoords"], m0["indices"], m0["material_indices"], mats, camera, width,
                                   height, max(1, settings.multiSample), settings.maxDepth, 1, 1,
                                   textures=textures, material_textures=mat_tex, meshes=meshes,
                                   mesh_material_offsets=offsets, instances=instances)
        warnings = [w for w in (info.warnings or b"").decode(errors="replace").split("\n") if w]
        return SceneFile(scene, camera, settings, sky, names(info.mesh_names, info.mesh_count),
                         names(info.instance_names, info.instance_count), material_names, warnings)
    finally:
        lib.tr_scene_file_free(h)


def write_model_cache(path, positions, indices, material_indices, materials, material_names, normals=None,
                      texcoords=None, texture_paths=None):
    """The reference's model cache format (ModelFile.cpp SaveToCache) for one mesh; texture_paths:
    optional (materials, 13) paths ('' for none) of the texture-enabled properties."""
    lib = _abi.load_library()
    pos = np.ascontiguousarray(positions, np.float32)
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
    uv = None if texcoords is None else np.ascontiguousarray(texcoords, np.float32)
    idx = np.ascontiguousarray(indices, np.uint32)
    mid = np.ascontiguousarray(material_indices, np.uint32)
    mats = np.ascontiguousarray(materials, MATERIAL_DTYPE)
    mesh = _abi.MeshDesc(pos.ctypes.data, None if nrm is None else nrm.ctypes.data,
                         None if uv is None else uv.ctypes.data, pos.shape[0], idx.shape[0], idx.ctypes.data,
                         mid.ctypes.data)
    name_arr = (C.c_char_p * len(material_names))(*[n.encode() for n in material_names])
    tex_arr = None
    if texture_paths is not None:
        flat = [(p or "").encode() for row in texture_paths for p in row]
        tex_arr = (C.c_char_p * len(flat))(*flat)
    _check(lib, lib.tr_model_cache_write(os.fsencode(path), C.byref(mesh), mats.ctypes.data, name_arr, tex_arr,
                                         mats.shape[0]), "tr_model_cache_write")


def write_texture_cache(path, texels: np.ndarray):
    """The reference's texture cache format (TextureFile.cpp SaveToCache): (H, W, 4) texels."""
    lib = _abi.load_library()
    t = np.ascontiguousarray(texels, np.float16)
    assert t.ndim == 3 and t.shape[2] == 4
    _check(lib, lib.tr_texture_cache_write(os.fsencode(path), t.shape[1], t.shape[0], t.ctypes.data),
           "tr_texture_cache_write")
