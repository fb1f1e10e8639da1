"""ctypes binding of libwfpt.so (the C ABI declared in include/wfpt.h).

The library is the only compute path: if it is missing the import fails
with an error that says how to build it; nothing falls back to host code.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libwfpt.so"

c_void_p = C.c_void_p
c_u32 = C.c_uint32
c_u64 = C.c_uint64
c_int = C.c_int
c_float = C.c_float
c_size_t = C.c_size_t
P_u32 = C.POINTER(C.c_uint32)
P_i32 = C.POINTER(C.c_int32)
P_f32 = C.POINTER(C.c_float)
P_size = C.POINTER(C.c_size_t)

WFPT_OK = 0
STATUS_NAMES = {
    0: "WFPT_OK",
    1: "WFPT_ERR_INVALID_ARGUMENT",
    2: "WFPT_ERR_CUDA",
    3: "WFPT_ERR_OUT_OF_MEMORY",
    4: "WFPT_ERR_TIMEOUT",
    5: "WFPT_ERR_UNSUPPORTED",
    6: "WFPT_ERR_SCRATCH_TOO_SMALL",
    7: "WFPT_ERR_DEVICE_BOUNDS",
}

BVH2_FP32 = 0
BVH8_Q8 = 1
MORTON_AILA32 = 0
MORTON_6D48 = 1
MORTON_6D64 = 2
PRIMARY_RAYS = 0
SHADOW_RAYS = 1
PATH_RAYS = 2


class WfptError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class RendererConfig(C.Structure):
    _fields_ = [
        ("ray_type", c_int),
        ("num_primary_samples", c_int),
        ("num_shadow_samples", c_int),
        ("shadow_radius", c_float),
        ("recursion_depth", c_int),
        ("key_value", c_float),
        ("white_point", c_float),
        ("russian_roulette", c_int),
        ("sort_shadow_rays", c_int),
        ("reorder_shadow_rays", c_int),
        ("sort_path_rays", c_int),
        ("reorder_path_rays", c_int),
        ("morton_kind", c_int),
        ("bvh_kind", c_int),
        ("albedo", c_float),
        ("use_graph", c_int),
        ("path_sort_skip", c_int),
        ("shadow_overlap", c_int),
        ("primary_bvh_kind", c_int),
        ("timing", c_int),
        ("accumulate_fp64", c_int),
    ]


class Camera(C.Structure):
    _fields_ = [
        ("position", c_float * 3),
        ("rotation_deg", c_float * 3),
        ("fov_deg", c_float),
        ("znear", c_float),
        ("zfar", c_float),
    ]


class SortLog(C.Structure):
    _fields_ = [
        ("ray_count", c_u64),
        ("morton_ms", c_float),
        ("sort_ms", c_float),
        ("reorder_ms", c_float),
        ("trace_sort_ms", c_float),
        ("trace_ms", c_float),
    ]


class RenderStats(C.Structure):
    _fields_ = [
        ("num_primary_rays", c_u64),
        ("num_shadow_rays", c_u64),
        ("num_path_rays", c_u64),
        ("path_rays_per_bounce", c_u32 * 8),
        ("shadow_hits_per_pass", c_u32 * 9),
        ("frame_ms", c_float),
        ("timed", c_int),
        ("primary_trace_ms", c_float),
        ("shadow_trace_ms", c_float),
        ("path_trace_ms", c_float),
        ("shadow_sort_logs", SortLog * 9),
        ("path_sort_logs", SortLog * 8),
        ("shadow_batch_slots", c_int),
    ]


class Request(C.Structure):
    _fields_ = [
        ("scene", c_void_p),
        ("geometries", c_void_p),
        ("light", c_float * 3),
        ("background", c_float * 3),
        ("camera", Camera),
        ("width", c_int),
        ("height", c_int),
        ("config", RendererConfig),
        ("pixels", c_void_p),
        ("frame_pixels", c_void_p),
    ]


class SceneInfo(C.Structure):
    _fields_ = [
        ("num_triangles", c_u32),
        ("num_geometries", c_u32),
        ("bvh2_nodes", c_u32),
        ("bvh8_nodes", c_u32),
        ("bounds_min", c_float * 3),
        ("bounds_max", c_float * 3),
        ("build_ms", C.c_double),
    ]


# name -> (restype, argtypes)
_SIGS = {
    "wfpt_abi_version": (c_int, []),
    "wfpt_status_string": (C.c_char_p, [c_int]),
    "wfpt_last_error_message": (C.c_char_p, []),
    "wfpt_device_status": (c_int, [P_u32]),
    "wfpt_kernel_launch_count": (c_u64, []),
    "wfpt_tune_set": (c_int, [C.c_char_p, C.c_int64]),
    "wfpt_tune_get": (c_int, [C.c_char_p, C.POINTER(C.c_int64)]),
    "wfpt_trace_counters": (c_int, [C.POINTER(c_u64), c_int]),
    "wfpt_pixel_table": (c_int, [c_int, c_int, c_void_p, c_void_p]),
    "wfpt_camera_screen_to_world": (c_int, [P_f32, P_f32, c_float, c_float, c_float, c_float, P_f32]),
    "wfpt_init_seeds": (c_int, [c_void_p, c_u32, c_int, c_void_p]),
    "wfpt_raygen_primary": (c_int, [P_f32, c_void_p, c_void_p, P_f32, c_int, c_int, c_int, c_float, c_void_p]),
    "wfpt_morton": (c_int, [c_void_p, c_u32, c_void_p, P_f32, P_f32, c_int, c_void_p, c_void_p, c_void_p]),
    "wfpt_sort_scratch_bytes": (c_size_t, [c_u32, c_int]),
    "wfpt_sort_pairs": (c_int, [c_void_p, c_void_p, c_u32, c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "wfpt_reorder": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_u32, c_void_p, c_void_p]),
    "wfpt_selftest_wait_timeout": (c_int, [c_int]),
    "wfpt_reorder_records": (c_int, [c_void_p, c_void_p, c_void_p, c_u32, c_void_p, c_void_p, c_void_p, c_u32, c_void_p,
                                     c_void_p]),
    "wfpt_raygen_shadow": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, P_f32, c_float, c_int,
                                   c_int, c_void_p, c_int, c_void_p]),
    "wfpt_raygen_path_scratch_bytes": (c_size_t, [c_u32]),
    "wfpt_raygen_path": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p, c_u32, c_void_p, c_int, c_float, c_void_p, c_size_t, c_void_p]),
    "wfpt_raygen_path_static": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p, c_u32, c_void_p, c_int, c_float, c_void_p]),
    "wfpt_reconstruct_smooth": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, P_f32, P_f32,
                                        c_u32, c_void_p, c_int, c_void_p]),
    "wfpt_reconstruct_shadow": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p,
                                        c_int, c_int, c_void_p]),
    "wfpt_count_hits": (c_int, [c_void_p, c_u32, c_void_p, c_void_p, c_void_p]),
    "wfpt_interpolate_colors": (c_int, [c_void_p, c_void_p, c_u32, c_int, c_float, c_float, c_void_p]),
    "wfpt_interpolate_colors_fp64": (c_int, [c_void_p, c_void_p, c_void_p, c_u32, c_int, c_float, c_float,
                                             c_void_p]),
    "wfpt_fill_u32": (c_int, [c_void_p, c_u32, c_size_t, c_void_p]),
    "wfpt_scene_create": (c_int, [c_void_p, c_u32, c_void_p, c_u32, c_void_p, c_u32, c_int, C.POINTER(c_void_p)]),
    "wfpt_scene_create_device": (c_int, [c_void_p, c_u32, c_void_p, c_u32, c_void_p, c_u32, c_int, c_void_p,
                                         C.POINTER(c_void_p)]),
    "wfpt_scene_destroy": (None, [c_void_p]),
    "wfpt_scene_get_info": (c_int, [c_void_p, C.POINTER(SceneInfo)]),
    "wfpt_scene_export_bvh2": (c_int, [c_void_p, c_void_p, P_size, c_void_p, P_size]),
    "wfpt_scene_export_bvh8": (c_int, [c_void_p, c_void_p, P_size, c_void_p, P_size]),
    "wfpt_trace": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_u32, c_void_p, c_int, c_void_p]),
    "wfpt_trace_sort": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_u32, c_void_p, P_f32, P_f32, c_int, c_int,
                                c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                c_size_t, c_void_p]),
    "wfpt_generate_scene":(c_int, [c_int, c_u64, c_u32, c_void_p, c_void_p, P_u32, c_void_p, P_u32]),
    "wfpt_renderer_config_default": (None, [C.POINTER(RendererConfig)]),
    "wfpt_renderer_create": (c_int, [C.POINTER(RendererConfig), C.POINTER(c_void_p)]),
    "wfpt_renderer_destroy": (None, [c_void_p]),
    "wfpt_renderer_set_config": (c_int, [c_void_p, C.POINTER(RendererConfig)]),
    "wfpt_renderer_set_scene": (c_int, [c_void_p, c_void_p, c_void_p, P_f32, P_f32, P_f32, P_f32]),
    "wfpt_renderer_reset_frame_index": (None, [c_void_p]),
    "wfpt_renderer_render": (c_int, [c_void_p, C.POINTER(Camera), c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "wfpt_renderer_get_stats": (c_int, [c_void_p, C.POINTER(RenderStats)]),
    "wfpt_batch_create": (c_int, [C.POINTER(Request), c_u32, c_int, C.POINTER(c_void_p)]),
    "wfpt_batch_destroy": (None, [c_void_p]),
    "wfpt_batch_render": (c_int, [c_void_p, C.POINTER(Camera), c_void_p]),
    "wfpt_batch_get_stats": (c_int, [c_void_p, c_u32, C.POINTER(RenderStats)]),
    "wfpt_batch_kernels": (c_u64, [c_void_p]),
    "wfpt_batch_reset_frame_index": (None, [c_void_p]),
}

EXPORTED = tuple(_SIGS)

_lib = None


def load() -> C.CDLL:
    """Loads libwfpt.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -m vulkanwavefrontpathtracer_gb300.build` "
            "(the CUDA library is the only compute path)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != WFPT_OK:
        msg = load().wfpt_last_error_message().decode(errors="replace")
        raise WfptError(status, msg)


def fvec(values, n: int | None = None):
    vals = list(values)
    if n is not None and len(vals) != n:
        raise ValueError(f"expected {n} floats, got {len(vals)}")
    return (c_float * len(vals))(*[float(v) for v in vals])
