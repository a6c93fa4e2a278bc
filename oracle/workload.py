"""The benchmark's synthetic scenes and camera UBOs for the CPU baseline
(TEST INFRASTRUCTURE).

oracle/_build/libworkload.so is the library's own host-only generator
(xvk_ray_gb300/csrc/scene_gen.cpp: xr_scene_cornell, xr_scene_procedural,
xr_camera_ubo, xr_params_default) built by oracle/Makefile on its own, so the CPU baseline renders
exactly the benchmark's scene and camera path without loading libxr.so.  The
ctypes structures come from xvk_ray_gb300._lib, whose import loads nothing.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from xvk_ray_gb300 import _lib as L
from xvk_ray_gb300.api import Scene

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libworkload.so"
_lib = None


def load():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
        lib = C.CDLL(str(LIB))
        P, u32 = C.c_void_p, C.c_uint32
        lib.xr_scene_cornell.restype, lib.xr_scene_cornell.argtypes = C.c_int32, [C.POINTER(L.XrSceneData)]
        lib.xr_scene_procedural.restype = C.c_int32
        lib.xr_scene_procedural.argtypes = [C.POINTER(L.XrProceduralDesc), C.POINTER(L.XrSceneData)]
        lib.xr_params_default.restype, lib.xr_params_default.argtypes = None, [C.POINTER(L.XrParams), u32, u32]
        lib.xr_camera_ubo.restype = C.c_int32
        lib.xr_camera_ubo.argtypes = [C.POINTER(L.XrCamera), u32, u32, P, u32, u32, u32, u32,
                                      C.POINTER(L.XrUniformBufferObject)]
        _lib = lib
    return _lib


def _check(status: int, what: str) -> None:
    if status != 0:
        raise RuntimeError(f"workload generator: {what} failed with status {status}")


def _generate(fn, *args) -> Scene:
    d = L.XrSceneData()
    _check(fn(*args, C.byref(d)), "scene size")
    v = np.zeros((d.vertex_count, 9), np.float32)
    i = np.zeros(d.index_count, np.uint32)
    m = np.zeros((d.material_count, 8), np.float32)
    d.vertices, d.indices, d.materials = v.ctypes.data, i.ctypes.data, m.ctypes.data
    _check(fn(*args, C.byref(d)), "scene")
    cam = L.XrCamera()
    C.memmove(C.byref(cam), C.byref(d.camera), C.sizeof(cam))
    return Scene(v, i, m, np.zeros((1, 2), np.uint32), cam)


def cornell() -> Scene:
    return _generate(load().xr_scene_cornell)


def procedural(seed: int = 1, n_objects: int = 4096, n_lights: int = 16, extent: float = 40.0,
               sphere_subdiv: int = 2) -> Scene:
    desc = L.XrProceduralDesc(seed, n_objects, n_lights, extent, sphere_subdiv)
    return _generate(load().xr_scene_procedural, C.byref(desc))


def camera_ubo(cam, width: int, height: int, prev, frame: int, bounces: int, sky: bool = False,
               reuse: bool = True) -> "L.XrUniformBufferObject":
    out = L.XrUniformBufferObject()
    _check(load().xr_camera_ubo(C.byref(cam), width, height, C.addressof(prev) if prev is not None else None, frame,
                                bounces, 1 if sky else 0, 1 if reuse else 0, C.byref(out)), "camera")
    return out


def params_default(width: int, height: int, **kw) -> "L.XrParams":
    """xr_params_default: the benchmark's corrected-pipeline settings."""
    p = L.XrParams()
    load().xr_params_default(C.byref(p), width, height)
    for k, v in kw.items():
        setattr(p, k, v)
    return p
