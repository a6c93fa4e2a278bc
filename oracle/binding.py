"""ctypes binding of oracle/_build/liboracle.so (see oracle/xr_oracle.h).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

BUF_SAMPLES, BUF_TEMPORAL, BUF_SPATIAL, BUF_HDR, BUF_LDR, BUF_PT, BUF_GBUF_POS, BUF_MOTION, BUF_WRITTEN = range(9)

_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            import subprocess
            subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
        lib = C.CDLL(str(LIB))
        P, u32 = C.c_void_p, C.c_uint32
        sig = {
            "or_init_random_seed": (u32, [u32, u32, u32, u32]),
            "or_random_sequence": (None, [u32, u32, P, P]),
            "or_sincos": (None, [P, u32, P, P]),
            "or_oct_roundtrip": (None, [P, u32, u32, P, P]),
            "or_scene_create": (P, [P, u32, P, u32, P, u32]),
            "or_scene_destroy": (None, [P]),
            "or_trace": (None, [P, P, u32, C.c_int, P, P, P]),
            "or_renderer_create": (P, [P, P]),
            "or_renderer_destroy": (None, [P]),
            "or_render_frame": (C.c_int, [P, P]),
            "or_set_samples": (C.c_int, [P, P, P]),
            "or_end_frame": (C.c_int, [P]),
            "or_run_pass": (C.c_int, [P, P, C.c_int]),
            "or_read": (C.c_size_t, [P, C.c_int, P, C.c_size_t]),
            "or_write_temporal": (C.c_int, [P, P, C.c_size_t]),
            "or_pt_reference": (C.c_int, [P, P, P, u32, u32, P]),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype, f.argtypes = r, a
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data if a is not None and a.size else None


def init_random_seed(x, y, w, frame) -> int:
    return load().or_init_random_seed(x, y, w, frame)


def random_sequence(state: int, n: int):
    u = np.empty(n, np.uint32)
    f = np.empty(n, np.float32)
    load().or_random_sequence(state, n, _p(u), _p(f))
    return u, f


def sincos(a: np.ndarray):
    a = np.ascontiguousarray(a, np.float32)
    s = np.empty_like(a)
    c = np.empty_like(a)
    load().or_sincos(_p(a), a.size, _p(s), _p(c))
    return s, c


def oct_roundtrip(n: np.ndarray, bits: int):
    n = np.ascontiguousarray(n, np.float32).reshape(-1, 3)
    out = np.empty_like(n)
    codes = np.empty(n.shape[0], np.uint32)
    load().or_oct_roundtrip(_p(n), n.shape[0], bits, _p(out), _p(codes))
    return out, codes


class OracleScene:
    def __init__(self, vertices: np.ndarray, global_indices: np.ndarray, materials: np.ndarray):
        self._v = np.ascontiguousarray(vertices, np.float32)
        self._i = np.ascontiguousarray(global_indices, np.uint32)
        self._m = np.ascontiguousarray(materials, np.float32)
        self.h = load().or_scene_create(_p(self._v), self._v.shape[0], _p(self._i), self._i.size // 3, _p(self._m),
                                        self._m.shape[0])

    @staticmethod
    def from_scene(scene) -> "OracleScene":
        return OracleScene(scene.vertices, scene.global_indices(), scene.materials)

    def trace(self, rays: np.ndarray, any_hit: bool = False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        bary = np.empty((n, 2), np.float32)
        load().or_trace(self.h, _p(rays), n, 1 if any_hit else 0, _p(prim), _p(t), _p(bary))
        return prim, t, bary

    def close(self):
        if self.h:
            load().or_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _bytes_of(struct) -> C.c_void_p:
    return C.cast(C.byref(struct), C.c_void_p)


class OracleRenderer:
    """State of one oracle render (reservoirs, G-buffers) across frames."""

    def __init__(self, scene: OracleScene, params):
        self.scene = scene
        self.params = params
        self.W, self.H = params.width, params.height
        self.h = load().or_renderer_create(scene.h, _bytes_of(params))

    def render(self, ubo) -> None:
        load().or_render_frame(self.h, _bytes_of(ubo))

    def set_samples(self, words: np.ndarray, ubo) -> None:
        w = np.ascontiguousarray(words, np.uint32)
        load().or_set_samples(self.h, _p(w), _bytes_of(ubo))

    def end_frame(self) -> None:
        load().or_end_frame(self.h)

    def run_pass(self, ubo, pass_id: int) -> None:
        load().or_run_pass(self.h, _bytes_of(ubo), pass_id)

    def write_temporal(self, words: np.ndarray) -> None:
        w = np.ascontiguousarray(words, np.uint32)
        assert load().or_write_temporal(self.h, _p(w), w.nbytes) == 0

    def read(self, which: int) -> np.ndarray:
        n = load().or_read(self.h, which, None, 0)
        raw = np.empty(n, np.uint8)
        load().or_read(self.h, which, _p(raw), n)
        if which == BUF_SAMPLES:
            return raw.view(np.uint32).reshape(-1, 24)
        if which in (BUF_TEMPORAL, BUF_SPATIAL):
            return raw.view(np.uint32).reshape(-1, 28)
        if which in (BUF_HDR, BUF_PT, BUF_GBUF_POS):
            return raw.view(np.float32).reshape(-1, 4)
        if which == BUF_LDR:
            return raw.reshape(-1, 4)
        if which == BUF_MOTION:
            return raw.view(np.float32).reshape(-1, 2)
        return raw.view(np.uint32)

    def close(self):
        if self.h:
            load().or_renderer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pt_reference(scene: OracleScene, params, ubo, frame0: int, spp: int) -> np.ndarray:
    out = np.empty((params.width * params.height, 3), np.float64)
    load().or_pt_reference(scene.h, _bytes_of(params), _bytes_of(ubo), frame0, spp, _p(out))
    return out
