"""Host-side mirror of the reference renderer's per-stage interface over the C ABI.

``DeviceRenderer`` follows Tracer::DeviceRenderer (Tracer/Renderer/DeviceRenderer.h:21-67):
RenderFrame(kernelSettings, renderMode, renderFlags), Reset, SetCamera, Resize,
Statistics, SampleCount, Resolution, Accumulator/ColorBuffer, PickRay; ``UpdateScene``
follows Renderer::UpdateScene (Tracer/Renderer/Renderer.h:49). Where the
reference calls FatalError -> exit (Tracer/CUDA/CudaError.cpp:13-25) these
methods raise ``TracerError`` with the C status.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import TR_FLAG_REFERENCE_SAMPLING, TR_FLAG_WRITE_AOVS  # noqa: F401
from .scenes import MATERIAL_DTYPE, CameraSpec, Scene


class TracerError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {_abi.STATUS.get(status, status)}{': ' + detail if detail else ''}")


class RenderModes(enum.IntEnum):
    """Tracer/Common/CommonStructs.h:110-125; PathTracing is the hot path, the other modes run the
    reference's other shade kernels (tr_set_render_mode)."""

    AmbientOcclusion = 0
    AmbientOcclusionShading = 1
    Bitangent = 2
    GeometricNormal = 3
    MaterialID = 4
    MaterialProperty = 5
    ObjectID = 6
    PathTracing = 7
    ShadingNormal = 8
    Tangent = 9
    TextureCoordinate = 10
    Wireframe = 11
    ZDepth = 12


@dataclass
class KernelSettings:
    """KernelSettings (Tracer/Common/CommonStructs.h:145-153) plus the knobs the reference hard-wires.

    Defaults follow Renderer::DefaultSettings (Tracer/Renderer/Renderer.cpp:255-266)."""

    multiSample: int = 1
    maxDepth: int = 16
    seed: int = 0
    aoDist: float = 1.0
    zDepthMax: float = 1.0
    rayEpsilon: float = 1e-3
    rrStart: int = 1           # PathTracing.h:149 (pathLength > 0)
    flags: int = 0
    maxColor: float = 10.0     # gMaxColorIntensity, CudaUtility.h:91
    traversalStepLimit: int = 0  # bound on BVH node visits per ray (0: 2^22); no reference counterpart

    def to_c(self) -> _abi.KernelSettings:
        return _abi.KernelSettings(self.multiSample, self.maxDepth, self.seed & 0xFFFFFFFF, self.rayEpsilon,
                                   min(self.rrStart, 0xFFFFFFFF), self.flags, self.maxColor,
                                   self.traversalStepLimit)


@dataclass
class SkySettings:
    """Tracer::Sky (Tracer/Renderer/Sky.h:16-67) with its defaults: the Preetham sky seen by
    paths that leave the scene (SampleSky, CudaSky.h:105-156)."""

    enabled: bool = True
    drawSun: bool = True
    sunDir: tuple = (0.0, 1.0, 0.0)
    sunAngularDiameter: float = 32.0   # arc minutes
    sunIntensity: float = 1000.0
    turbidity: float = 4.0
    selectionBias: float = 1.0

    def to_c(self) -> _abi.SkyDesc:
        return _abi.SkyDesc(int(bool(self.enabled)), int(bool(self.drawSun)), (C.c_float * 3)(*self.sunDir),
                            self.sunAngularDiameter, self.sunIntensity, self.turbidity, self.selectionBias)


@dataclass(frozen=True)
class RayPickResult:
    """RayPickResult (CommonStructs.h:132-141); instIx and primIx are 0xFFFFFFFF on a miss."""

    rayOrigin: tuple
    instIx: int
    rayDir: tuple
    primIx: int
    tmax: float

    @property
    def hit(self) -> bool:
        return self.primIx != 0xFFFFFFFF


def camera_to_c(cam: CameraSpec) -> _abi.Camera:
    side, up, fwd = cam.basis()
    c = _abi.Camera()
    c.position[:] = [float(x) for x in np.asarray(cam.position, np.float32)]
    c.side[:] = [float(x) for x in side]
    c.up[:] = [float(x) for x in up]
    c.forward[:] = [float(x) for x in fwd]
    c.aperture = cam.aperture
    c.distortion = cam.distortion
    c.focal_dist = cam.focal_dist
    c.fov = cam.fov
    c.bokeh_side_count = cam.bokeh_side_count
    c.bokeh_rotation = cam.bokeh_rotation
    return c


class SceneDescHolder:
    """Keeps the numpy arrays of a Scene alive while the C structs point at them."""

    def __init__(self, scene: Scene, leaf_size: int = 0, build_threads: int = 0):
        self.scene = scene
        self.pos = np.ascontiguousarray(scene.positions, np.float32)
        self.nrm = None if scene.normals is None else np.ascontiguousarray(scene.normals, np.float32)
        self.uv = None if scene.texcoords is None else np.ascontiguousarray(scene.texcoords, np.float32)
        self.idx = np.ascontiguousarray(scene.indices, np.uint32)
        self.mat = np.ascontiguousarray(scene.material_indices, np.uint32)
        self.mats = np.ascontiguousarray(scene.materials, MATERIAL_DTYPE)
        self.mesh = _abi.MeshDesc(
            self.pos.ctypes.data,
            None if self.nrm is None else self.nrm.ctypes.data,
            None if self.uv is None else self.uv.ctypes.data,
            self.pos.shape[0],
            self.idx.shape[0],
            self.idx.ctypes.data,
            self.mat.ctypes.data,
        )
        self.desc = _abi.SceneDesc(C.pointer(self.mesh), C.cast(self.mats.ctypes.data, C.POINTER(_abi.MaterialDesc)),
                                   self.mats.shape[0], leaf_size, build_threads, 0)
        if scene.material_textures is not None and len(scene.textures) > 0:
            self.tex_arrays = [np.ascontiguousarray(t, np.float16) for t in scene.textures]
            self.tex = (_abi.TextureDesc * len(self.tex_arrays))()
            for i, t in enumerate(self.tex_arrays):
                assert t.ndim == 3 and t.shape[2] == 4, "textures are (H, W, 4) RGBA"
                self.tex[i] = _abi.TextureDesc(t.shape[1], t.shape[0], t.ctypes.data)
            self.mat_tex = np.ascontiguousarray(scene.material_textures, np.uint32)
            self.desc.texture_count = len(self.tex_arrays)
            self.desc.textures = C.cast(self.tex, C.c_void_p)
            self.desc.material_textures = self.mat_tex.ctypes.data
        inst = getattr(scene, "instances", None)
        if inst is not None:
            # two-level scene: meshes placed by instances
            self.meshes = (_abi.MeshDesc * len(scene.meshes))()
            self.mesh_arrays = []
            for i, m in enumerate(scene.meshes):
                arrs = [np.ascontiguousarray(m["positions"], np.float32),
                        None if m.get("normals") is None else np.ascontiguousarray(m["normals"], np.float32),
                        None if m.get("texcoords") is None else np.ascontiguousarray(m["texcoords"], np.float32),
                        np.ascontiguousarray(m["indices"], np.uint32),
                        np.ascontiguousarray(m["material_indices"], np.uint32)]
                self.mesh_arrays.append(arrs)
                self.meshes[i] = _abi.MeshDesc(arrs[0].ctypes.data, None if arrs[1] is None else arrs[1].ctypes.data,
                                               None if arrs[2] is None else arrs[2].ctypes.data, arrs[0].shape[0],
                                               arrs[3].shape[0], arrs[3].ctypes.data, arrs[4].ctypes.data)
            self.offsets = np.ascontiguousarray(scene.mesh_material_offsets, np.uint32)
            self.inst = (_abi.InstanceDesc * len(inst))()
            for i, (mesh_ix, xf) in enumerate(inst):
                self.inst[i].mesh = int(mesh_ix)
                self.inst[i].transform[:] = [float(x) for x in np.asarray(xf, np.float32).reshape(12)]
            self.desc.instance_count = len(inst)
            self.desc.meshes = C.cast(self.meshes, C.POINTER(_abi.MeshDesc))
            self.desc.mesh_material_offsets = self.offsets.ctypes.data
            self.desc.instances = C.cast(self.inst, C.POINTER(_abi.InstanceDesc))
            self.desc.mesh_count = len(scene.meshes)

    def ptr(self):
        return C.byref(self.desc)


class DeviceRenderer:
    def __init__(self, device: int = 0):
        self._lib = _abi.load_library()
        self._ctx = C.c_void_p()
        cfg = _abi.Config(device, _abi.TR_ABI_VERSION)
        st = self._lib.tr_create(C.byref(cfg), C.byref(self._ctx))
        if st != 0:
            raise TracerError(st, "tr_create")
        self._scene_holder = None
        self._settings = KernelSettings()
        self._resolution = (0, 0)

    # ------------------------------------------------------------------ plumbing
    def _check(self, st: int, where: str):
        if st != 0:
            detail = self._lib.tr_last_error(self._ctx).decode(errors="replace") if self._ctx else ""
            raise TracerError(st, where, detail)

    def close(self):
        if self._ctx:
            self._lib.tr_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._ctx

    # ------------------------------------------------------------------ scene / camera / settings
    def UpdateScene(self, scene: Scene, leaf_size: int = 0, build_threads: int = 0):
        holder = SceneDescHolder(scene, leaf_size, build_threads)
        self._check(self._lib.tr_scene_upload(self._ctx, holder.ptr()), "tr_scene_upload")
        self._scene_holder = holder

    def SceneInfo(self) -> dict:
        info = _abi.SceneInfo()
        self._check(self._lib.tr_get_scene_info(self._ctx, C.byref(info)), "tr_get_scene_info")
        return {f: (list(getattr(info, f)) if f == "scene_bounds" else getattr(info, f)) for f, _ in info._fields_}

    def SetCamera(self, cam: CameraSpec):
        self._check(self._lib.tr_set_camera(self._ctx, C.byref(camera_to_c(cam))), "tr_set_camera")

    def SetSettings(self, settings: KernelSettings):
        self._check(self._lib.tr_set_settings(self._ctx, C.byref(settings.to_c())), "tr_set_settings")
        self._settings = settings

    def Resize(self, resolution):
        w, h = resolution
        self._check(self._lib.tr_resize(self._ctx, int(w), int(h)), "tr_resize")
        self._resolution = (int(w), int(h))

    def Reset(self):
        self._check(self._lib.tr_reset(self._ctx), "tr_reset")

    # ------------------------------------------------------------------ rendering
    def RenderFrame(self, kernelSettings: KernelSettings | None = None,
                    renderMode: RenderModes = RenderModes.PathTracing, renderFlags: int = 0, stream: int = 0,
                    use_graph: bool = False):
        if kernelSettings is not None:
            self.SetSettings(kernelSettings)
        ks = kernelSettings or self._settings
        self._check(self._lib.tr_set_render_mode(self._ctx, int(renderMode), int(renderFlags), float(ks.aoDist),
                                                 float(ks.zDepthMax)), "tr_set_render_mode")
        self._check(self._lib.tr_render_frame(self._ctx, C.c_void_p(stream or None), int(use_graph)),
                    "tr_render_frame")

    def RenderSamples(self, spp: int, stream: int = 0, use_graph: bool = True):
        """tr_render_samples: spp samples per pixel (a multiple of multi_sample) added to the
        accumulation as one continuous wavefront (same samples as spp / multi_sample frames)."""
        self._check(self._lib.tr_render_samples(self._ctx, C.c_void_p(stream or None), int(spp), int(use_graph)),
                    "tr_render_samples")

    def BeginFrame(self, stream: int = 0):
        self._check(self._lib.tr_begin_frame(self._ctx, C.c_void_p(stream or None)), "tr_begin_frame")

    def Generate(self, stream: int = 0):
        self._check(self._lib.tr_generate(self._ctx, C.c_void_p(stream or None)), "tr_generate")

    def Extend(self, bounce: int, stream: int = 0):
        self._check(self._lib.tr_extend(self._ctx, C.c_void_p(stream or None), bounce), "tr_extend")

    def Shade(self, bounce: int, stream: int = 0):
        self._check(self._lib.tr_shade(self._ctx, C.c_void_p(stream or None), bounce), "tr_shade")

    def Connect(self, bounce: int, stream: int = 0):
        self._check(self._lib.tr_connect(self._ctx, C.c_void_p(stream or None), bounce), "tr_connect")

    def Finalize(self, stream: int = 0):
        self._check(self._lib.tr_finalize(self._ctx, C.c_void_p(stream or None)), "tr_finalize")

    def UpdateMaterials(self, materials: np.ndarray):
        """tr_update_materials: new material table for the uploaded scene (no BVH rebuild)."""
        mats = np.ascontiguousarray(materials, MATERIAL_DTYPE)
        self._check(self._lib.tr_update_materials(self._ctx, C.cast(mats.ctypes.data, C.POINTER(_abi.MaterialDesc)),
                                                  mats.shape[0]), "tr_update_materials")

    def AdjointFrame(self, pixel_grad_ptr: int, scale: float, param_grad_ptr: int, stream: int = 0):
        """tr_adjoint_frame on device buffers: pixel gradient (float4 per pixel) -> (materials, 9) gradient."""
        self._check(self._lib.tr_adjoint_frame(self._ctx, C.c_void_p(stream or None), C.c_void_p(pixel_grad_ptr),
                                               scale, C.c_void_p(param_grad_ptr)), "tr_adjoint_frame")

    def Tuning(self) -> dict:
        t = _abi.Tuning()
        self._check(self._lib.tr_get_tuning(self._ctx, C.byref(t)), "tr_get_tuning")
        return {f: getattr(t, f) for f, _ in t._fields_ if f != "reserved"}

    def SetTuning(self, **kw):
        t = _abi.Tuning()
        for k, v in kw.items():
            setattr(t, k, int(v))
        self._check(self._lib.tr_set_tuning(self._ctx, C.byref(t)), "tr_set_tuning")

    def Autotune(self, stream: int = 0, skip_bvh: bool = False, samples: bool = False) -> dict:
        """tr_autotune: times launch shapes (and BVH leaf sizes) on the current frame setup; with
        samples=True on continuous renders of 4 x multi_sample samples per pixel (RenderSamples)."""
        rep = _abi.TuneReport()
        flags = (_abi.TR_TUNE_SKIP_BVH if skip_bvh else 0) | (_abi.TR_TUNE_SAMPLES if samples else 0)
        self._check(self._lib.tr_autotune(self._ctx, C.c_void_p(stream or None), flags, C.byref(rep)),
                    "tr_autotune")
        chosen = {f: getattr(rep.chosen, f) for f, _ in rep.chosen._fields_ if f != "reserved"}
        return {"chosen": chosen, "frame_ms_default": rep.frame_ms_default, "frame_ms_tuned": rep.frame_ms_tuned,
                "trials": rep.trials}

    def SetSky(self, sky: SkySettings | None):
        """Scene::GetSky settings (None disables the sky, the state a context starts in)."""
        d = sky.to_c() if sky is not None else None
        self._check(self._lib.tr_set_sky(self._ctx, C.byref(d) if d is not None else None), "tr_set_sky")

    def PickRay(self, pixelIndex, stream: int = 0) -> RayPickResult:
        """DeviceRenderer::PickRay (DeviceRenderer.cpp:71-92): what the camera ray through pixel
        (x, y) hits first; waits for the result."""
        x, y = pixelIndex
        r = _abi.RayPickResult()
        self._check(self._lib.tr_pick_ray(self._ctx, C.c_void_p(stream or None), int(x), int(y), C.byref(r)),
                    "tr_pick_ray")
        return RayPickResult(tuple(r.ray_origin), int(r.inst_ix), tuple(r.ray_dir), int(r.prim_ix), float(r.tmax))

    def Synchronize(self, stream: int = 0):
        self._check(self._lib.tr_synchronize(self._ctx, C.c_void_p(stream or None)), "tr_synchronize")

    # ------------------------------------------------------------------ results
    def Statistics(self) -> dict:
        s = _abi.Statistics()
        self._check(self._lib.tr_get_statistics(self._ctx, C.byref(s)), "tr_get_statistics")
        out = {}
        for f, _ in s._fields_:
            v = getattr(s, f)
            out[f] = list(v) if f in ("extend_rays", "shadow_rays", "hit_rays") else v
        return out

    def SampleCount(self) -> int:
        return int(self.Statistics()["sample_count"])

    def Resolution(self):
        return self._resolution

    def Buffers(self) -> dict:
        b = _abi.Buffers()
        self._check(self._lib.tr_get_buffers(self._ctx, C.byref(b)), "tr_get_buffers")
        return {
            "path_state": [b.path_state[0], b.path_state[1]],
            "hits": b.hits,
            "shadow": b.shadow,
            "radiance": b.radiance,
            "accumulator": b.accumulator,
            "albedo": b.albedo,
            "normals": b.normals,
            "colors": b.colors,
            "counters": b.counters,
            "capacity": b.capacity,
            "width": b.width,
            "height": b.height,
        }

    def ColorBuffer(self, out: np.ndarray | None = None, stream: int = 0) -> np.ndarray:
        w, h = self._resolution
        if out is None:
            out = np.empty((h, w, 4), np.float32)
        self._check(self._lib.tr_download_image(self._ctx, C.c_void_p(stream or None), out.ctypes.data, out.nbytes),
                    "tr_download_image")
        return out

    def Accumulator(self) -> np.ndarray:
        w, h = self._resolution
        out = np.empty((h, w, 4), np.float32)
        self._check(self._lib.tr_download_accumulator(self._ctx, None, out.ctypes.data, out.nbytes),
                    "tr_download_accumulator")
        return out

    def read_device(self, ptr: int, dtype, count: int) -> np.ndarray:
        out = np.empty(count, dtype)
        self._check(self._lib.tr_copy_from_device(self._ctx, out.ctypes.data, C.c_void_p(ptr), out.nbytes),
                    "tr_copy_from_device")
        return out

    def write_device(self, ptr: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr)
        self._check(self._lib.tr_copy_to_device(self._ctx, C.c_void_p(ptr), a.ctypes.data, a.nbytes),
                    "tr_copy_to_device")


def settings_for(scene: Scene, multi_sample: int = 1, reference: bool = False, seed: int | None = None,
                 aovs: bool = False) -> KernelSettings:
    flags = (TR_FLAG_REFERENCE_SAMPLING if reference else 0) | (TR_FLAG_WRITE_AOVS if aovs else 0)
    return KernelSettings(multiSample=multi_sample, maxDepth=scene.max_depth,
                          seed=scene.seed if seed is None else seed, rrStart=1 if reference else scene.rr_start,
                          flags=flags)


class BatchRenderer:
    """Many independent scenes rendered by one continuous wavefront (tr_batch_*): each item
    is (scene, spp) with the scene's own camera and resolution; pool_paths path slots (0: the
    library's default) are kept full with the items' samples."""

    def __init__(self, scenes, spp=None, pool_paths: int = 0, device: int = 0):
        self._lib = _abi.load_library()
        self._b = C.c_void_p()
        self.scenes = list(scenes)
        self.spp = [s.spp for s in self.scenes] if spp is None else [int(x) for x in spp]
        holders = [SceneDescHolder(s) for s in self.scenes]
        items = (_abi.BatchItem * len(self.scenes))()
        for i, (s, h) in enumerate(zip(self.scenes, holders)):
            items[i].scene = C.pointer(h.desc)
            items[i].camera = camera_to_c(s.camera)
            items[i].width = s.width
            items[i].height = s.height
            items[i].spp = self.spp[i]
        cfg = _abi.Config(device, _abi.TR_ABI_VERSION)
        st = self._lib.tr_batch_create(C.byref(cfg), items, len(self.scenes), int(pool_paths), C.byref(self._b))
        if st != 0:
            raise TracerError(st, "tr_batch_create")

    def _check(self, st: int, where: str):
        if st != 0:
            raise TracerError(st, where, self._lib.tr_batch_last_error(self._b).decode(errors="replace"))

    def close(self):
        if self._b:
            self._lib.tr_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def Render(self, settings: KernelSettings, stream: int = 0, use_graph: bool = True):
        c = settings.to_c()
        self._check(self._lib.tr_batch_render(self._b, C.c_void_p(stream or None), C.byref(c), int(use_graph)),
                    "tr_batch_render")

    def Info(self) -> dict:
        i = _abi.BatchInfo()
        self._check(self._lib.tr_batch_get_info(self._b, C.byref(i)), "tr_batch_get_info")
        return {f: getattr(i, f) for f, _ in i._fields_ if f != "reserved"}

    def Statistics(self) -> dict:
        s = _abi.BatchStatistics()
        self._check(self._lib.tr_batch_get_statistics(self._b, C.byref(s)), "tr_batch_get_statistics")
        return {f: getattr(s, f) for f, _ in s._fields_}

    def Image(self, item: int, out: np.ndarray | None = None, stream: int = 0) -> np.ndarray:
        s = self.scenes[item]
        if out is None:
            out = np.empty((s.height, s.width, 4), np.float32)
        self._check(self._lib.tr_batch_download(self._b, C.c_void_p(stream or None), item, out.ctypes.data,
                                                out.nbytes), "tr_batch_download")
        return out
