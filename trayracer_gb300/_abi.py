"""ctypes view of the C ABI declared in include/trayracer.h."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

TR_MAX_DEPTH = 16
TR_ABI_VERSION = 3
TR_FLAG_REFERENCE_SAMPLING = 1 << 0
TR_FLAG_WRITE_AOVS = 1 << 1
TR_FLAG_REFERENCE_DRAW_RTL = 1 << 2
TR_FLAG_COUNT_TRAVERSAL = 1 << 3

TR_CLOSURE_LAMBERT = 0
TR_CLOSURE_DIFFUSE = 1
TR_CLOSURE_DISNEY = 2

STATUS = {
    0: "TR_OK",
    1: "TR_ERR_INVALID_ARGUMENT",
    2: "TR_ERR_OUT_OF_MEMORY",
    3: "TR_ERR_CUDA",
    4: "TR_ERR_NO_SCENE",
    5: "TR_ERR_NOT_READY",
    6: "TR_ERR_LIMIT",
    7: "TR_ERR_DEVICE_FAULT",
}


class KernelSettings(C.Structure):
    _fields_ = [
        ("multi_sample", C.c_uint32),
        ("max_depth", C.c_uint32),
        ("seed", C.c_uint32),
        ("ray_epsilon", C.c_float),
        ("rr_start", C.c_uint32),
        ("flags", C.c_uint32),
        ("max_color", C.c_float),
        ("traversal_step_limit", C.c_uint32),
    ]


class Camera(C.Structure):
    _fields_ = [
        ("position", C.c_float * 3),
        ("side", C.c_float * 3),
        ("up", C.c_float * 3),
        ("forward", C.c_float * 3),
        ("aperture", C.c_float),
        ("distortion", C.c_float),
        ("focal_dist", C.c_float),
        ("fov", C.c_float),
        ("bokeh_side_count", C.c_int32),
        ("bokeh_rotation", C.c_float),
    ]


class MaterialDesc(C.Structure):
    _fields_ = [
        ("diffuse", C.c_float * 3),
        ("emissive", C.c_float * 3),
        ("metallic", C.c_float),
        ("subsurface", C.c_float),
        ("specular", C.c_float),
        ("roughness", C.c_float),
        ("specular_tint", C.c_float),
        ("anisotropic", C.c_float),
        ("sheen", C.c_float),
        ("sheen_tint", C.c_float),
        ("clearcoat", C.c_float),
        ("clearcoat_gloss", C.c_float),
        ("closure", C.c_uint32),
    ]


class MeshDesc(C.Structure):
    _fields_ = [
        ("positions", C.c_void_p),
        ("normals", C.c_void_p),
        ("texcoords", C.c_void_p),
        ("vertex_count", C.c_uint32),
        ("triangle_count", C.c_uint32),
        ("indices", C.c_void_p),
        ("material_indices", C.c_void_p),
    ]


class InstanceDesc(C.Structure):
    _fields_ = [
        ("mesh", C.c_uint32),
        ("reserved", C.c_uint32),
        ("transform", C.c_float * 12),
    ]


TR_PROP_COUNT = 13
TR_PROP_DIFFUSE = 3
TR_PROP_EMISSIVE = 4
TR_PROP_METALLIC = 5
TR_PROP_NORMAL = 6
TR_PROP_ROUGHNESS = 7
TR_NO_TEXTURE = 0xFFFFFFFF


class SceneDesc(C.Structure):
    _fields_ = [
        ("mesh", C.POINTER(MeshDesc)),
        ("materials", C.POINTER(MaterialDesc)),
        ("material_count", C.c_uint32),
        ("bvh_leaf_size", C.c_uint32),
        ("build_threads", C.c_uint32),
        ("instance_count", C.c_uint32),
        ("meshes", C.POINTER(MeshDesc)),
        ("mesh_material_offsets", C.c_void_p),
        ("instances", C.POINTER(InstanceDesc)),
        ("mesh_count", C.c_uint32),
        ("texture_count", C.c_uint32),
        ("textures", C.c_void_p),
        ("material_textures", C.c_void_p),
    ]


class TextureDesc(C.Structure):
    """tr_texture_desc: RGBA binary16 texels."""

    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("texels", C.c_void_p)]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("abi_version", C.c_uint32)]


class Statistics(C.Structure):
    _fields_ = [
        ("path_count", C.c_uint64),
        ("primary_path_count", C.c_uint64),
        ("secondary_path_count", C.c_uint64),
        ("deep_path_count", C.c_uint64),
        ("shadow_ray_count", C.c_uint64),
        ("extend_rays", C.c_uint32 * TR_MAX_DEPTH),
        ("shadow_rays", C.c_uint32 * TR_MAX_DEPTH),
        ("render_time_ms", C.c_float),
        ("generate_time_ms", C.c_float),
        ("extend_time_ms", C.c_float),
        ("shade_time_ms", C.c_float),
        ("connect_time_ms", C.c_float),
        ("finalize_time_ms", C.c_float),
        ("sample_count", C.c_uint32),
        ("device_error", C.c_uint32),
        ("traversal_extend_nodes", C.c_uint64),
        ("traversal_extend_tris", C.c_uint64),
        ("traversal_connect_nodes", C.c_uint64),
        ("traversal_connect_tris", C.c_uint64),
        ("hit_rays", C.c_uint32 * TR_MAX_DEPTH),
        ("radiance_updates_shade", C.c_uint64),
        ("radiance_updates_connect", C.c_uint64),
        ("iterations", C.c_uint32),
        ("launches", C.c_uint32),
        ("hit_ray_count", C.c_uint64),
    ]


class SceneInfo(C.Structure):
    _fields_ = [
        ("triangle_count", C.c_uint32),
        ("light_count", C.c_uint32),
        ("material_count", C.c_uint32),
        ("bvh_node_count", C.c_uint32),
        ("device_bytes", C.c_uint64),
        ("light_energy", C.c_float),
        ("build_time_ms", C.c_float),
        ("upload_time_ms", C.c_float),
        ("scene_bounds", C.c_float * 6),
    ]


class Buffers(C.Structure):
    _fields_ = [
        ("path_state", C.c_void_p * 2),
        ("hits", C.c_void_p),
        ("shadow", C.c_void_p),
        ("radiance", C.c_void_p),
        ("accumulator", C.c_void_p),
        ("albedo", C.c_void_p),
        ("normals", C.c_void_p),
        ("colors", C.c_void_p),
        ("counters", C.c_void_p),
        ("capacity", C.c_uint64),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("bvh_leaf_size", C.c_uint32),
        ("refill_below", C.c_uint32),
        ("extend_blocks_per_sm", C.c_uint32),
        ("connect_blocks_per_sm", C.c_uint32),
        ("shade_waves", C.c_uint32),
        ("sort_hits", C.c_uint32),
        ("traversal_threads", C.c_uint32),
        ("shade_threads", C.c_uint32),
        ("bvh_nodes", C.c_uint32),
    ]


class SkyDesc(C.Structure):
    """tr_sky_desc (Tracer::Sky settings, Sky.h:16-67)."""

    _fields_ = [
        ("enabled", C.c_uint32),
        ("draw_sun", C.c_uint32),
        ("sun_dir", C.c_float * 3),
        ("sun_angular_diameter", C.c_float),
        ("sun_intensity", C.c_float),
        ("turbidity", C.c_float),
        ("selection_bias", C.c_float),
    ]


class RayPickResult(C.Structure):
    """tr_ray_pick_result (RayPickResult, CommonStructs.h:132-141)."""

    _fields_ = [
        ("ray_origin", C.c_float * 3),
        ("inst_ix", C.c_uint32),
        ("ray_dir", C.c_float * 3),
        ("prim_ix", C.c_uint32),
        ("tmax", C.c_float),
    ]


class TuneReport(C.Structure):
    _fields_ = [
        ("chosen", Tuning),
        ("frame_ms_default", C.c_float),
        ("frame_ms_tuned", C.c_float),
        ("trials", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


TR_TUNE_SKIP_BVH = 1 << 0
TR_TUNE_SAMPLES = 1 << 1


class BatchItem(C.Structure):
    _fields_ = [
        ("scene", C.POINTER(SceneDesc)),
        ("camera", Camera),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("spp", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class BatchInfo(C.Structure):
    _fields_ = [
        ("item_count", C.c_uint32),
        ("round_count", C.c_uint32),
        ("path_count", C.c_uint64),
        ("pixel_count", C.c_uint64),
        ("triangle_count", C.c_uint64),
        ("device_bytes", C.c_uint64),
        ("pool_paths", C.c_uint32),
        ("reserved", C.c_uint32),
        ("build_time_ms", C.c_float),
        ("upload_time_ms", C.c_float),
    ]


class BatchStatistics(C.Structure):
    _fields_ = [
        ("extend_rays", C.c_uint64),
        ("shadow_rays", C.c_uint64),
        ("hit_rays", C.c_uint64),
        ("render_time_ms", C.c_float),
        ("device_error", C.c_uint32),
        ("traversal_extend_nodes", C.c_uint64),
        ("traversal_extend_tris", C.c_uint64),
        ("traversal_connect_nodes", C.c_uint64),
        ("traversal_connect_tris", C.c_uint64),
        ("iterations", C.c_uint32),
        ("launches", C.c_uint32),
    ]


# name -> (restype, argtypes) for every function include/trayracer.h declares
class SceneFileInfo(C.Structure):
    """tr_scene_file_info."""

    _fields_ = [
        ("scene", C.POINTER(SceneDesc)),
        ("camera", Camera),
        ("camera_target", C.c_float * 3),
        ("camera_up", C.c_float * 3),
        ("settings", KernelSettings),
        ("ao_dist", C.c_float),
        ("z_depth_max", C.c_float),
        ("sky", SkyDesc),
        ("mesh_count", C.c_uint32),
        ("instance_count", C.c_uint32),
        ("mesh_names", C.POINTER(C.c_char_p)),
        ("instance_names", C.POINTER(C.c_char_p)),
        ("material_names", C.POINTER(C.c_char_p)),
        ("warnings", C.c_char_p),
    ]


_V = C.c_void_p
_U = C.c_uint32
FUNCTIONS = {
    "tr_create": (C.c_int, [C.POINTER(Config), C.POINTER(_V)]),
    "tr_destroy": (C.c_int, [_V]),
    "tr_status_string": (C.c_char_p, [C.c_int]),
    "tr_last_error": (C.c_char_p, [_V]),
    "tr_scene_upload": (C.c_int, [_V, C.POINTER(SceneDesc)]),
    "tr_get_scene_info": (C.c_int, [_V, C.POINTER(SceneInfo)]),
    "tr_set_camera": (C.c_int, [_V, C.POINTER(Camera)]),
    "tr_set_settings": (C.c_int, [_V, C.POINTER(KernelSettings)]),
    "tr_resize": (C.c_int, [_V, _U, _U]),
    "tr_reset": (C.c_int, [_V]),
    "tr_begin_frame": (C.c_int, [_V, _V]),
    "tr_generate": (C.c_int, [_V, _V]),
    "tr_extend": (C.c_int, [_V, _V, _U]),
    "tr_shade": (C.c_int, [_V, _V, _U]),
    "tr_connect": (C.c_int, [_V, _V, _U]),
    "tr_finalize": (C.c_int, [_V, _V]),
    "tr_render_frame": (C.c_int, [_V, _V, C.c_int32]),
    "tr_render_samples": (C.c_int, [_V, _V, _U, C.c_int32]),
    "tr_synchronize": (C.c_int, [_V, _V]),
    "tr_get_statistics": (C.c_int, [_V, C.POINTER(Statistics)]),
    "tr_get_buffers": (C.c_int, [_V, C.POINTER(Buffers)]),
    "tr_download_image": (C.c_int, [_V, _V, _V, C.c_uint64]),
    "tr_download_accumulator": (C.c_int, [_V, _V, _V, C.c_uint64]),
    "tr_copy_from_device": (C.c_int, [_V, _V, _V, C.c_uint64]),
    "tr_copy_to_device": (C.c_int, [_V, _V, _V, C.c_uint64]),
    "tr_trace_host": (C.c_int, [C.POINTER(SceneDesc), _V, _V, _U, C.c_float, C.c_int32, _V, _V]),
    "tr_update_materials": (C.c_int, [_V, C.POINTER(MaterialDesc), _U]),
    "tr_adjoint_frame": (C.c_int, [_V, _V, _V, C.c_float, _V]),
    "tr_render_frame_noalloc": (C.c_int, [_V, _V, _V, _V, _U]),
    "tr_set_render_mode": (C.c_int, [_V, _U, _U, C.c_float, C.c_float]),
    "tr_pick_ray": (C.c_int, [_V, _V, C.c_int32, C.c_int32, C.POINTER(RayPickResult)]),
    "tr_set_sky": (C.c_int, [_V, C.POINTER(SkyDesc)]),
    "tr_scene_file_load": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(_V)]),
    "tr_scene_file_get_info": (C.c_int, [_V, C.POINTER(SceneFileInfo)]),
    "tr_scene_file_free": (C.c_int, [_V]),
    "tr_scene_file_last_error": (C.c_char_p, []),
    "tr_model_cache_write": (C.c_int, [C.c_char_p, C.POINTER(MeshDesc), _V, _V, _V, _U]),
    "tr_texture_cache_write": (C.c_int, [C.c_char_p, _U, _U, _V]),
    "tr_get_tuning": (C.c_int, [_V, C.POINTER(Tuning)]),
    "tr_set_tuning": (C.c_int, [_V, C.POINTER(Tuning)]),
    "tr_autotune": (C.c_int, [_V, _V, _U, C.POINTER(TuneReport)]),
    "tr_batch_create": (C.c_int, [C.POINTER(Config), C.POINTER(BatchItem), _U, C.c_uint64, C.POINTER(_V)]),
    "tr_batch_destroy": (C.c_int, [_V]),
    "tr_batch_last_error": (C.c_char_p, [_V]),
    "tr_batch_get_info": (C.c_int, [_V, C.POINTER(BatchInfo)]),
    "tr_batch_render": (C.c_int, [_V, _V, C.POINTER(KernelSettings), C.c_int32]),
    "tr_batch_get_statistics": (C.c_int, [_V, C.POINTER(BatchStatistics)]),
    "tr_batch_get_colors": (C.c_int, [_V, _U, C.POINTER(_V)]),
    "tr_batch_download": (C.c_int, [_V, _V, _U, _V, C.c_uint64]),
}

LIB_PATH = Path(__file__).resolve().parent / "libtrayracer.so"
_lib = None


def load_library() -> C.CDLL:
    """Loads libtrayracer.so; raises when it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')"
        )
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in FUNCTIONS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
