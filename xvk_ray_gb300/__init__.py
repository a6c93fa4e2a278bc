"""GB300-native ReSTIR GI frame pipeline (drop-in for XVK_Ray's ReSTIR GI render pass).

The compute path is libxr.so (hand-written CUDA for sm_103a) behind the C ABI in
include/xr.h; this package binds it with ctypes.  Importing the package does
not need a GPU; creating a Renderer does.
"""
from . import _lib
from ._lib import XrError, load
from .api import (CACHE_SAMPLE_DTYPE, INSTANCE_DTYPE, Cache, PinnedBuffer, Renderer, Scene, cache_params_default,
                  camera_ubo, pack_instances, params_default, params_reference, ubo_bytes)
from .path_tracer import PathTracer, UserSettings

__all__ = ["XrError", "load", "Renderer", "Scene", "PinnedBuffer", "Cache", "CACHE_SAMPLE_DTYPE", "cache_params_default",
           "INSTANCE_DTYPE", "pack_instances", "camera_ubo", "params_default",
           "params_reference", "ubo_bytes", "PathTracer", "UserSettings", "_lib"]
