"""Python bindings of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs import this package: it is the checker and the timed CPU baseline, never
part of the product path.

``Oracle``    - oracle/liboracle.so, the restated reference algorithm (float for
                parity, double for the FP64 image).
``Reference`` - oracle/_ref/libtrref.so, the reference's own raygen and shade
                kernels compiled as host C++ (only where the reference sources
                were present at build time).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from trayracer_gb300 import _abi
from trayracer_gb300.renderer import SceneDescHolder, camera_to_c
from trayracer_gb300.scenes import CameraSpec, Scene

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libtrref.so"

_P = C.c_void_p
_U = C.c_uint32


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


class Oracle:
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not ORACLE_LIB.exists():
                from . import build as _b

                _b.build_oracle()
            lib = C.CDLL(str(ORACLE_LIB))
            lib.orc_scene_create.restype = _P
            lib.orc_scene_create.argtypes = [_P]
            lib.orc_scene_destroy.argtypes = [_P]
            lib.orc_light_count.restype = _U
            lib.orc_light_count.argtypes = [_P]
            lib.orc_light_energy.restype = C.c_float
            lib.orc_light_energy.argtypes = [_P, C.c_int]
            lib.orc_generate.argtypes = [_P, _P, _P, _U, _U, _U, _U, _U, _P, _P, _P]
            lib.orc_trace_closest.argtypes = [_P, _P, _P, _U, C.c_float, _P]
            lib.orc_trace_ray.restype = C.c_int
            lib.orc_trace_ray.argtypes = [_P, _P, _P, C.c_float, C.c_float, C.c_int, _P, _P, _P, _P, _P]
            lib.orc_pick_ray.argtypes = [_P, _P, _P, _U, _U, C.c_int32, C.c_int32, _P]
            lib.orc_set_sky.argtypes = [_P, _P]
            lib.orc_texture_sample.argtypes = [_P, _U, C.c_float, C.c_float, _P]
            lib.orc_ties.restype = _U
            lib.orc_ties.argtypes = [_P, _P, _P, C.c_float, C.c_float, C.c_float, _P, _U, _P]
            lib.orc_trace_any.argtypes = [_P, _P, _P, _U, C.c_float, _P]
            lib.orc_shade.argtypes = [_P, _P, _U, _U, _U, _U, _U, _P, _P, _P, _P, _P, _P, _P, _P, _P]
            lib.orc_shade_fp64.argtypes = [_P, _P, _U, _U, _U, _U, _U, _P, _P, _P, _P, _P, _P, _P, _P, _P]
            lib.orc_render.restype = C.c_int
            lib.orc_render.argtypes = [_P, _P, _P, _U, _U, _U, _U, _U, C.c_int, C.c_int, _P, _P, _P]
            lib.orc_counter_rng.argtypes = [_U, _U, _U, _U, _U, _P]
            lib.orc_reference_rng.argtypes = [_U, _U, _U, _P]
            lib.orc_set_reference_draw_order.argtypes = [C.c_int]
            lib.orc_closure.argtypes = [C.c_int, C.c_int, C.c_int, _P, _P]
            lib.orc_closure_value_grad.argtypes = [_P, _U, _P, _P, _P]
            lib.orc_adjoint.restype = C.c_int
            lib.orc_adjoint.argtypes = [_P, _P, _P, _U, _U, _U, _P, C.c_float, C.c_int, C.c_int, _P]
            cls._lib = lib
        return cls._lib

    def __init__(self, scene: Scene):
        self.lib()
        self.scene = scene
        self._holder = SceneDescHolder(scene)
        self._s = self._lib.orc_scene_create(C.addressof(self._holder.desc))
        if not self._s:
            raise RuntimeError("orc_scene_create failed")

    def __del__(self):
        if getattr(self, "_s", None) and self._lib is not None:
            self._lib.orc_scene_destroy(self._s)
            self._s = None

    @property
    def light_count(self) -> int:
        return int(self._lib.orc_light_count(self._s))

    def light_energy(self, total: bool = True) -> float:
        return float(self._lib.orc_light_energy(self._s, int(total)))

    def generate(self, cam: CameraSpec, settings, width, height, sample_count, first, n):
        O = np.empty((n, 4), np.float32)
        D = np.empty((n, 4), np.float32)
        T = np.empty((n, 4), np.float32)
        cc = camera_to_c(cam)
        st = settings.to_c()
        self._lib.orc_generate(self._s, C.addressof(cc), C.addressof(st), width, height, sample_count, first, n,
                               _ptr(O), _ptr(D), _ptr(T))
        return O, D, T

    def texture_sample(self, texture: int, u: float, v: float) -> np.ndarray:
        """tex2D<float4> of one of the scene's textures at (u, v), as the texture unit filters it."""
        out = np.zeros(4, np.float32)
        self._lib.orc_texture_sample(self._s, int(texture), float(u), float(v), _ptr(out))
        return out

    def set_sky(self, sky):
        """Sky seen by paths that leave the scene (a trayracer_gb300 SkySettings, or None: disabled)."""
        self._sky = sky.to_c() if sky is not None else None
        self._lib.orc_set_sky(self._s, C.addressof(self._sky) if self._sky is not None else None)

    def pick_ray(self, cam: CameraSpec, settings, width, height, x, y) -> np.ndarray:
        """RayPickResult of pixel (x, y) as 9 float32 words (instIx, primIx as bit patterns)."""
        out = np.zeros(9, np.float32)
        cc = camera_to_c(cam)
        st = settings.to_c()
        self._lib.orc_pick_ray(self._s, C.addressof(cc), C.addressof(st), width, height, int(x), int(y), _ptr(out))
        return out

    def trace_closest(self, O: np.ndarray, D: np.ndarray, tmin: float) -> np.ndarray:
        O = np.ascontiguousarray(O, np.float32)
        D = np.ascontiguousarray(D, np.float32)
        hits = np.empty((O.shape[0], 4), np.uint32)
        self._lib.orc_trace_closest(self._s, _ptr(O), _ptr(D), O.shape[0], tmin, _ptr(hits))
        return hits

    def ties(self, O, D, tmin: float, t: float, rel: float = 1e-6, max_out: int = 16, with_instances=False):
        """Triangles hit at t within rel (mesh-local indices; with_instances: (instance, triangle) pairs)."""
        o = np.ascontiguousarray(O[:3], np.float32)
        d = np.ascontiguousarray(D[:3], np.float32)
        prims = np.zeros(max_out, np.uint32)
        insts = np.zeros(max_out, np.uint32)
        n = self._lib.orc_ties(self._s, _ptr(o), _ptr(d), tmin, t, rel, _ptr(prims), max_out, _ptr(insts))
        k = min(n, max_out)
        if with_instances:
            return [(int(i), int(p)) for i, p in zip(insts[:k], prims[:k])]
        return [int(p) for p in prims[:k]]

    def trace_any(self, O: np.ndarray, L: np.ndarray, eps: float) -> np.ndarray:
        O = np.ascontiguousarray(O, np.float32)
        L = np.ascontiguousarray(L, np.float32)
        occ = np.empty(O.shape[0], np.uint8)
        self._lib.orc_trace_any(self._s, _ptr(O), _ptr(L), O.shape[0], eps, _ptr(occ))
        return occ

    def shade(self, settings, bounce, sample_count, width, height, O, D, T, hits, fp64=False):
        n = O.shape[0]
        O = np.ascontiguousarray(O, np.float32)
        D = np.ascontiguousarray(D, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        hits = np.ascontiguousarray(hits, np.uint32)
        ext = np.zeros((n, 3, 4), np.float32)
        sh = np.zeros((n, 3, 4), np.float32)
        ev = np.zeros(n, np.uint8)
        sv = np.zeros(n, np.uint8)
        rad = np.zeros((n, 4), np.float32)
        st = settings.to_c()
        fn = self._lib.orc_shade_fp64 if fp64 else self._lib.orc_shade
        fn(self._s, C.addressof(st), bounce, sample_count, width, height, n, _ptr(O), _ptr(D), _ptr(T), _ptr(hits),
           _ptr(ext), _ptr(ev), _ptr(sh), _ptr(sv), _ptr(rad))
        return ext, ev.astype(bool), sh, sv.astype(bool), rad

    def render(self, cam: CameraSpec, settings, width, height, frames=1, first_pixel=0, pixel_count=None,
               use_double=False, threads=0, want_paths=False):
        """Accumulator (float64, (pixels, 4)) of `frames` frames; optional per-path radiance of the last frame."""
        if pixel_count is None:
            pixel_count = width * height - first_pixel
        acc = np.zeros((pixel_count, 4), np.float64)
        paths = np.zeros((settings.multiSample, pixel_count, 4), np.float64) if want_paths else None
        counts = np.zeros(2, np.uint64)
        cc = camera_to_c(cam)
        st = settings.to_c()
        self._lib.orc_render(self._s, C.addressof(cc), C.addressof(st), width, height, frames, first_pixel,
                             pixel_count, int(use_double), threads, _ptr(acc), _ptr(paths), _ptr(counts))
        return acc, paths, (int(counts[0]), int(counts[1]))

    def adjoint(self, cam: CameraSpec, settings, width, height, sample_count, pixel_grad, scale=1.0,
                use_double=True, threads=0):
        """Path-replay gradient (material_count, 9) of the frame with sample_count."""
        pg = np.ascontiguousarray(pixel_grad, np.float32).reshape(-1, 4)
        grads = np.zeros((self.scene.materials.shape[0], 9), np.float64)
        cc = camera_to_c(cam)
        st = settings.to_c()
        rc = self._lib.orc_adjoint(self._s, C.addressof(cc), C.addressof(st), width, height, sample_count,
                                   _ptr(pg), scale, int(use_double), threads, _ptr(grads))
        if rc != 0:
            raise RuntimeError("the adjoint differentiates the default sampling mode only")
        return grads

    def closure_value_grad(self, material: int, wo, wi) -> np.ndarray:
        """(3, 7): per channel the closure value and its 6 parameter derivatives."""
        o = np.ascontiguousarray(wo, np.float32)
        i = np.ascontiguousarray(wi, np.float32)
        out = np.zeros((3, 7), np.float64)
        self._lib.orc_closure_value_grad(self._s, material, _ptr(o), _ptr(i), _ptr(out))
        return out

    @classmethod
    def closure(cls, ctype: int, inputs: np.ndarray, reference: bool = True, use_double: bool = False):
        """Closure outputs (n, 14) for inputs (n, 31), layout of orc_closure."""
        inputs = np.ascontiguousarray(inputs, np.float32)
        out = np.zeros((inputs.shape[0], 14), np.float32)
        lib = cls.lib()
        for i in range(inputs.shape[0]):
            lib.orc_closure(ctype, int(reference), int(use_double), inputs[i].ctypes.data, out[i].ctypes.data)
        return out

    @classmethod
    def set_reference_draw_order(cls, right_to_left: bool):
        cls.lib().orc_set_reference_draw_order(int(right_to_left))

    @classmethod
    def counter_rng(cls, pixel, sample, bounce, seed, n):
        out = np.empty(n, np.float32)
        cls.lib().orc_counter_rng(pixel, sample, bounce, seed, n, _ptr(out))
        return out

    @classmethod
    def reference_rng(cls, v0, v1, n):
        out = np.empty(n, np.float32)
        cls.lib().orc_reference_rng(v0, v1, n, _ptr(out))
        return out


def reference_available() -> bool:
    return REF_LIB.exists()


class Reference:
    """The reference's own kernels run on the host (oracle/_ref/libtrref.so)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not REF_LIB.exists():
                raise RuntimeError("oracle/_ref/libtrref.so is not built (reference sources absent)")
            lib = C.CDLL(str(REF_LIB))
            lib.ref_create.restype = _P
            lib.ref_create.argtypes = [_P]
            lib.ref_destroy.argtypes = [_P]
            lib.ref_primary.argtypes = [_P, _P, _P, _U, _U, _U, _P, _P, _P]
            lib.ref_secondary.argtypes = [_P, _P, _P, _U, _U, _U, _U, _P, _P]
            lib.ref_shade.argtypes = [_P, _P, _P, _U, _U, _U, _U, _U, _P, _P, _P, _P, _P, _P, _P]
            lib.ref_shadow.argtypes = [_P, _P, _P, _U, _U, _U, _U, _P, _P]
            lib.ref_render_frame.argtypes = [_P, _P, _P, _U, _U, _U, _P, _P, _P]
            lib.ref_closure.argtypes = [C.c_int, _P, _P]
            lib.ref_rng.argtypes = [_U, _U, _U, _P]
            lib.ref_set_render_mode.argtypes = [_U, _U, C.c_float, C.c_float]
            lib.ref_pick_ray.argtypes = [_P, _P, _P, _U, _U, C.c_int32, C.c_int32, _P]
            lib.ref_set_sky.argtypes = [_P, _P]
            cls._lib = lib
        return cls._lib

    def __init__(self, scene: Scene):
        self.lib()
        self.scene = scene
        self._holder = SceneDescHolder(scene)
        self._c = self._lib.ref_create(C.addressof(self._holder.desc))

    @classmethod
    def closure(cls, ctype: int, inputs: np.ndarray) -> np.ndarray:
        inputs = np.ascontiguousarray(inputs, np.float32)
        out = np.zeros((inputs.shape[0], 14), np.float32)
        lib = cls.lib()
        for i in range(inputs.shape[0]):
            lib.ref_closure(ctype, inputs[i].ctypes.data, out[i].ctypes.data)
        return out

    @classmethod
    def rng(cls, v0: int, v1: int, n: int) -> np.ndarray:
        out = np.empty(n, np.float32)
        cls.lib().ref_rng(v0, v1, n, out.ctypes.data)
        return out

    def __del__(self):
        if getattr(self, "_c", None) and self._lib is not None:
            self._lib.ref_destroy(self._c)
            self._c = None

    @classmethod
    def set_render_mode(cls, mode: int, flags: int = 0, ao_dist: float = 1.0, z_depth_max: float = 1.0):
        """RenderModes value, MaterialPropertyIds flags, aoDist, zDepthMax for the following frames."""
        cls.lib().ref_set_render_mode(int(mode), int(flags), float(ao_dist), float(z_depth_max))

    def render_frame(self, cam: CameraSpec, settings, width, height, sample_count, accumulator):
        """One DeviceRenderer::RenderFrame; accumulator (H*W, 4) float32 is updated in place."""
        ext = np.zeros(16, np.uint32)
        sh = np.zeros(16, np.uint32)
        cc = camera_to_c(cam)
        st = settings.to_c()
        self._lib.ref_render_frame(self._c, C.addressof(cc), C.addressof(st), width, height, sample_count,
                                   _ptr(accumulator), _ptr(ext), _ptr(sh))
        return ext, sh

    def set_sky(self, sky):
        """The SkyData of a Tracer::Sky with these settings (None: disabled)."""
        self._sky = sky.to_c() if sky is not None else None
        self._lib.ref_set_sky(self._c, C.addressof(self._sky) if self._sky is not None else None)

    def pick_ray(self, cam: CameraSpec, settings, width, height, x, y) -> np.ndarray:
        """DeviceRenderer::PickRay through the RayPick raygen: RayPickResult as 9 float32 words."""
        out = np.zeros(9, np.float32)
        cc = camera_to_c(cam)
        st = settings.to_c()
        self._lib.ref_pick_ray(self._c, C.addressof(cc), C.addressof(st), width, height, int(x), int(y), _ptr(out))
        return out

    def primary(self, cam, settings, width, height, sample_count, accumulator):
        stride = width * height * settings.multiSample
        states = np.zeros((3, stride, 4), np.float32)
        hits = np.zeros((stride, 4), np.uint32)
        cc = camera_to_c(cam)
        st = settings.to_c()
        self._lib.ref_primary(self._c, C.addressof(cc), C.addressof(st), width, height, sample_count, _ptr(states),
                              _ptr(hits), _ptr(accumulator))
        return states, hits

    def secondary(self, cam, settings, width, height, sample_count, path_count, states, hits):
        cc = camera_to_c(cam)
        st = settings.to_c()
        self._lib.ref_secondary(self._c, C.addressof(cc), C.addressof(st), width, height, sample_count, path_count,
                                _ptr(states), _ptr(hits))

    def shade(self, cam, settings, width, height, sample_count, path_length, path_count, states, hits, shadow,
              accumulator):
        albedo = np.zeros((width * height, 4), np.float32)
        normals = np.zeros((width * height, 4), np.float32)
        counters = np.zeros(2, np.uint32)
        cc = camera_to_c(cam)
        st = settings.to_c()
        self._lib.ref_shade(self._c, C.addressof(cc), C.addressof(st), width, height, sample_count, path_length,
                            path_count, _ptr(states), _ptr(hits), _ptr(shadow), _ptr(accumulator), _ptr(albedo),
                            _ptr(normals), _ptr(counters))
        return int(counters[0]), int(counters[1])

    def shadow(self, cam, settings, width, height, sample_count, count, shadow, accumulator):
        cc = camera_to_c(cam)
        st = settings.to_c()
        self._lib.ref_shadow(self._c, C.addressof(cc), C.addressof(st), width, height, sample_count, count,
                             _ptr(shadow), _ptr(accumulator))
