"""ctypes binding of libxr.so (include/xr.h).

The library is the CUDA implementation; there is no other code path.  Loading
fails with an ImportError-style RuntimeError when the shared object has not
been built (run ``python -c "import __graft_entry__ as g; g.build()"``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libxr.so"

XR_OK = 0
XR_ERR_INVALID_ARGUMENT = 1
XR_ERR_CUDA = 2
XR_ERR_OUT_OF_MEMORY = 3
XR_ERR_STATE = 4
XR_ERR_OVERFLOW = 5
XR_ERR_TIMEOUT = 6
XR_ERR_UNSUPPORTED = 7

XR_MAT_LAMBERTIAN = 0
XR_MAT_METALLIC = 1
XR_MAT_DIFFUSE_LIGHT = 4
XR_MAT_PLASTIC = 5

XR_OUT_LDR8 = 0
XR_OUT_HDR = 1
XR_OUT_PT = 2

XR_BUF_SAMPLES = 0
XR_BUF_TEMPORAL = 1
XR_BUF_SPATIAL = 2


class XrVertex(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("normal", C.c_float * 3), ("tex_coord", C.c_float * 2),
                ("material_index", C.c_int32)]


class XrMaterial(C.Structure):
    _fields_ = [("base_color", C.c_float * 4), ("base_color_texture_index", C.c_int32), ("fuzziness", C.c_float),
                ("refraction_index", C.c_float), ("material_model", C.c_uint32)]


class XrMeshRange(C.Structure):
    _fields_ = [("index_offset", C.c_uint32), ("vertex_offset", C.c_uint32)]


class XrUniformBufferObject(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("view_prev", C.c_float * 16), ("projection", C.c_float * 16),
                ("projection_prev", C.c_float * 16), ("view_inverse", C.c_float * 16),
                ("projection_inverse", C.c_float * 16), ("spp", C.c_uint32),
                ("total_number_of_samples", C.c_uint32), ("number_of_bounces", C.c_uint32),
                ("random_seed", C.c_uint32), ("has_sky_box", C.c_uint32), ("reuse", C.c_uint32),
                ("current_frame", C.c_uint32)]


class XrParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("compat_reference", C.c_uint32),
                ("temporal_on", C.c_uint32), ("spatial_on", C.c_uint32), ("m_cap_temporal", C.c_uint32),
                ("m_cap_spatial", C.c_uint32), ("n_neighbours", C.c_uint32), ("radius_px", C.c_float),
                ("visibility", C.c_uint32), ("seed", C.c_uint32), ("write_pt", C.c_uint32),
                ("write_hdr", C.c_uint32)]


class XrDeviceDesc(C.Structure):
    _fields_ = [("device", C.c_int32), ("width", C.c_uint32), ("height", C.c_uint32)]


class XrStats(C.Structure):
    _fields_ = [("frames", C.c_uint32), ("error_flags", C.c_uint32), ("ms_initial", C.c_float),
                ("ms_temporal", C.c_float), ("ms_spatial", C.c_float), ("ms_frame", C.c_float),
                ("rays_traced", C.c_uint64), ("shadow_rays", C.c_uint64), ("bvh_nodes", C.c_uint32),
                ("bvh_triangles", C.c_uint32), ("bvh_depth", C.c_uint32), ("ms_bvh_build", C.c_float),
                ("query_rays", C.c_uint64), ("query_node_visits", C.c_uint64), ("query_tri_tests", C.c_uint64),
                ("nonfinite_rays", C.c_uint64), ("instances", C.c_uint32), ("tlas_nodes", C.c_uint32),
                ("ms_tlas_build", C.c_float), ("ms_refit", C.c_float)]


class XrInstance(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("reserved", C.c_uint32), ("object_to_world", C.c_float * 12)]


class XrCamera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("yaw_deg", C.c_float), ("pitch_deg", C.c_float),
                ("fov_deg", C.c_float)]


class XrSceneData(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("vertex_count", C.c_uint32), ("indices", C.c_void_p),
                ("index_count", C.c_uint32), ("materials", C.c_void_p), ("material_count", C.c_uint32),
                ("camera", XrCamera)]


class XrProceduralDesc(C.Structure):
    _fields_ = [("seed", C.c_uint32), ("n_objects", C.c_uint32), ("n_lights", C.c_uint32),
                ("extent", C.c_float), ("sphere_subdiv", C.c_uint32)]


class XrCacheParams(C.Structure):
    _fields_ = [("enabled", C.c_uint32), ("train", C.c_uint32), ("train_samples", C.c_uint32),
                ("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("seed", C.c_uint32)]


class XrCacheSample(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("normal", C.c_float * 3), ("wo", C.c_float * 3), ("albedo", C.c_float * 3),
                ("roughness", C.c_float), ("kind", C.c_uint32), ("target", C.c_float * 3), ("pixel", C.c_uint32)]


class XrCacheStats(C.Structure):
    _fields_ = [("steps", C.c_uint32), ("queries", C.c_uint32), ("train_samples", C.c_uint32), ("loss", C.c_float),
                ("ms_infer", C.c_float), ("ms_train", C.c_float), ("bounds_lo", C.c_float * 3),
                ("inv_extent", C.c_float)]


class XrTexture(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgba8", C.POINTER(C.c_uint8))]


class XrView(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32)]


class XrTuning(C.Structure):
    _fields_ = [("trace_ctas_per_sm", C.c_uint32), ("shade_ctas_per_sm", C.c_uint32), ("ms_per_frame", C.c_float),
                ("ms_default", C.c_float), ("configs_tried", C.c_uint32), ("refill_min", C.c_uint32),
                ("postpone_below", C.c_uint32), ("ray_bundle", C.c_uint32), ("temporal_block", C.c_uint32),
                ("spatial_block", C.c_uint32)]


XR_CACHE_MLP, XR_CACHE_GRID, XR_CACHE_MLP_GRAD, XR_CACHE_GRID_GRAD = 0, 1, 2, 3
XR_CACHE_MLP_M, XR_CACHE_MLP_V, XR_CACHE_GRID_M, XR_CACHE_GRID_V = 4, 5, 6, 7
XR_CACHE_QUERIES, XR_CACHE_TRAIN_RECORDS, XR_CACHE_ADAM_STEP = 8, 9, 10
XR_DEVFLAG_MMA_TIMEOUT = 8

assert C.sizeof(XrCacheParams) == 32 and C.sizeof(XrCacheSample) == 72 and C.sizeof(XrCacheStats) == 40
assert C.sizeof(XrVertex) == 36 and C.sizeof(XrMaterial) == 32
assert C.sizeof(XrUniformBufferObject) == 412 and C.sizeof(XrParams) == 52

# name -> (restype, argtypes)
_P = C.c_void_p
_u32 = C.c_uint32
_i32 = C.c_int32
_SIGS = {
    "xr_api_version": (_u32, []),
    "xr_last_error": (C.c_char_p, [_P]),
    "xr_params_default": (None, [C.POINTER(XrParams), _u32, _u32]),
    "xr_params_reference": (None, [C.POINTER(XrParams), _u32, _u32]),
    "xr_create": (_i32, [C.POINTER(XrDeviceDesc), C.POINTER(_P)]),
    "xr_destroy": (None, [_P]),
    "xr_upload_scene": (_i32, [_P, _P, _u32, _P, _u32, _P, _u32, _P, _u32]),
    "xr_build_bvh": (_i32, [_P]),
    "xr_set_params": (_i32, [_P, C.POINTER(XrParams)]),
    "xr_get_params": (_i32, [_P, C.POINTER(XrParams)]),
    "xr_render_frame": (_i32, [_P, C.POINTER(XrUniformBufferObject)]),
    "xr_read_output": (_i32, [_P, _u32, _P, C.c_size_t]),
    "xr_render_reference": (_i32, [_P, C.POINTER(XrUniformBufferObject), _u32, _u32, _P]),
    "xr_output_device_ptr": (_i32, [_P, _u32, C.POINTER(_P)]),
    "xr_read_output_async": (_i32, [_P, _P, C.c_size_t]),
    "xr_wait_output": (_i32, [_P]),
    "xr_sync": (_i32, [_P]),
    "xr_get_stats": (_i32, [_P, C.POINTER(XrStats)]),
    "xr_read_buffer": (_i32, [_P, _u32, _P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "xr_write_buffer": (_i32, [_P, _u32, _P, C.c_size_t]),
    "xr_run_pass": (_i32, [_P, C.POINTER(XrUniformBufferObject), _u32]),
    "xr_trace_rays": (_i32, [_P, _P, _u32, _i32, _P, _P, _P]),
    "xr_trace_rays_device": (_i32, [_P, _P, _u32, _i32, _P, _P, _P]),
    "xr_trace_rays_noalloc": (_i32, [_P, _P, _u32, _i32, _P, _P, _P]),
    "xr_camera_ubo": (_i32, [C.POINTER(XrCamera), _u32, _u32, C.POINTER(XrUniformBufferObject), _u32, _u32, _u32,
                             _u32, C.POINTER(XrUniformBufferObject)]),
    "xr_scene_cornell": (_i32, [C.POINTER(XrSceneData)]),
    "xr_scene_procedural": (_i32, [C.POINTER(XrProceduralDesc), C.POINTER(XrSceneData)]),
    "xr_event_record": (_i32, [_P, _u32]),
    "xr_event_elapsed": (_i32, [_P, _u32, _u32, C.POINTER(C.c_float)]),
    "xr_alloc_host": (_i32, [C.c_size_t, C.POINTER(_P)]),
    "xr_free_host": (None, [_P]),
    "xr_upload_textures": (_i32, [_P, _P, _u32]),
    "xr_png_unfilter": (_i32, [_P, _u32, _u32, _u32, _P]),
    "xr_upload_scenes": (_i32, [_P, _P, _u32]),
    "xr_set_instances": (_i32, [_P, _P, _u32]),
    "xr_get_instance_transforms": (_i32, [_P, _P, _u32]),
    "xr_update_vertices": (_i32, [_P, _u32, _P, _u32]),
    "xr_trace_rays_instanced": (_i32, [_P, _P, _u32, _i32, _P, _P, _P, _P]),
    "xr_set_views": (_i32, [_P, _P, _u32, C.POINTER(XrParams)]),
    "xr_render_views": (_i32, [_P, _P]),
    "xr_read_view_output": (_i32, [_P, _u32, _u32, _P, C.c_size_t]),
    "xr_render_reference_views": (_i32, [_P, _P, _u32, _u32, _P]),
    "xr_set_graphs": (_i32, [_P, C.c_int]),
    "xr_autotune": (_i32, [_P, _P, _u32, C.POINTER(XrTuning)]),
    "xr_set_tuning": (_i32, [_P, C.POINTER(XrTuning)]),
    "xr_cache_params_default": (None, [C.POINTER(XrCacheParams)]),
    "xr_cache_set_params": (_i32, [_P, C.POINTER(XrCacheParams)]),
    "xr_cache_get_params": (_i32, [_P, C.POINTER(XrCacheParams)]),
    "xr_cache_reset": (_i32, [_P, _u32]),
    "xr_cache_set_bounds": (_i32, [_P, _P, C.c_float]),
    "xr_cache_query": (_i32, [_P, _P, _u32, _P]),
    "xr_cache_train": (_i32, [_P, _P, _u32, C.c_int, C.POINTER(C.c_float)]),
    "xr_cache_step": (_i32, [_P]),
    "xr_cache_selftest_wait": (_i32, [_P, _u32]),
    "xr_cache_read": (_i32, [_P, C.c_int, _P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "xr_cache_write": (_i32, [_P, C.c_int, _P, C.c_size_t]),
    "xr_cache_get_stats": (_i32, [_P, C.POINTER(XrCacheStats)]),
}

EXPORTED = tuple(_SIGS)

_lib = None


def load() -> C.CDLL:
    """Loads libxr.so once; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first (xvk_ray_gb300._build)")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class XrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"xr status {status}: {message}")
        self.status = status


def check(status: int, ctx=None) -> None:
    if status != XR_OK:
        msg = load().xr_last_error(ctx)
        raise XrError(status, msg.decode() if msg else "")
