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
BUF_CACHE_QUERIES, BUF_CACHE_TRAIN = 9, 10

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
            "or_units_onb": (None, [P, u32, P]),
            "or_units_sample_hemisphere": (None, [P, u32, P]),
            "or_units_sample_bsdf": (None, [P, P, P, P, u32, P]),
            "or_units_update_list": (None, [P, P, u32, u32, P, P, P]),
            "or_units_merge_list": (None, [P, P, u32, u32, P, P, P]),
            "or_units_similar": (None, [P, P, u32, P]),
            "or_units_aces": (None, [P, u32, P]),
            "or_units_targets": (None, [P, P, P, u32, P]),
            "or_units_world_to_screen_uv": (None, [P, u32, P, P, P]),
            "or_units_neighbor_index": (None, [u32, u32, u32, u32, C.c_float, u32, u32, P]),
            "or_scene_create": (P, [P, u32, P, u32, P, u32]),
            "or_scene_destroy": (None, [P]),
            "or_scene_set_textures": (None, [P, P, u32, P]),
            "or_trace": (None, [P, P, u32, C.c_int, P, P, P]),
            "or_world_create": (P, [P, u32]),
            "or_world_set_instances": (C.c_int, [P, P, P, u32]),
            "or_world_transforms": (None, [P, P]),
            "or_world_update_vertices": (C.c_int, [P, u32, P, u32]),
            "or_trace_inst": (None, [P, P, u32, C.c_int, P, P, P, P]),
            "or_renderer_create": (P, [P, P]),
            "or_renderer_destroy": (None, [P]),
            "or_renderer_set_cache": (C.c_int, [P, C.c_int, u32, P]),
            "or_render_frame": (C.c_int, [P, P]),
            "or_set_samples": (C.c_int, [P, P, P]),
            "or_end_frame": (C.c_int, [P]),
            "or_run_pass": (C.c_int, [P, P, C.c_int]),
            "or_read": (C.c_size_t, [P, C.c_int, P, C.c_size_t]),
            "or_write_temporal": (C.c_int, [P, P, C.c_size_t]),
            "or_pt_reference": (C.c_int, [P, P, P, u32, u32, P]),
            "or_nrc_create": (P, [u32]),
            "or_nrc_destroy": (None, [P]),
            "or_nrc_set_bounds": (None, [P, P, C.c_float]),
            "or_nrc_params": (C.POINTER(C.c_float), [P, C.c_int, C.POINTER(C.c_size_t)]),
            "or_nrc_pack": (None, [P, u32, P]),
            "or_nrc_inputs": (None, [P, P, u32, P, C.c_int]),
            "or_nrc_infer": (None, [P, P, u32, P, C.c_int]),
            "or_nrc_backward": (C.c_double, [P, P, P, u32, C.c_int, C.c_int]),
            "or_nrc_loss": (C.c_double, [P, P, P, u32, C.c_int, C.c_int]),
            "or_nrc_adam": (None, [P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]),
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
        o = OracleScene(scene.vertices, scene.global_indices(), scene.materials)
        textures = getattr(scene, "textures", None) or []
        if textures:
            sizes = np.array([[t.shape[1], t.shape[0]] for t in textures], np.uint32)
            texels = np.concatenate([np.ascontiguousarray(t, np.uint8).reshape(-1) for t in textures])
            load().or_scene_set_textures(o.h, _p(sizes), len(textures), _p(texels))
        return o

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


class OracleWorld(OracleScene):
    """Scenes concatenated as xr_upload_scenes does, traced and rendered through
    instances (or_world_*); usable wherever an OracleScene is."""

    def __init__(self, scenes: "list[OracleScene]"):
        self._parts = list(scenes)   # keep the sources alive while copying
        arr = (C.c_void_p * len(scenes))(*[sc.h for sc in scenes])
        self.h = load().or_world_create(C.cast(arr, C.c_void_p), len(scenes))
        self._n_inst = 0

    def set_instances(self, instances) -> None:
        """instances: (scene index, 3x4 object-to-world) pairs."""
        n = len(instances)
        part = np.array([int(k) for k, _ in instances], np.uint32)
        m = np.array([np.asarray(x, np.float32).reshape(12) for _, x in instances], np.float32).reshape(n, 12)
        if load().or_world_set_instances(self.h, _p(part), _p(m), n) != 0:
            raise ValueError("bad instance list (unknown scene or singular transform)")
        self._n_inst = n

    def transforms(self) -> np.ndarray:
        out = np.empty((self._n_inst, 24), np.float32)
        if self._n_inst:
            load().or_world_transforms(self.h, _p(out))
        return out.reshape(self._n_inst, 2, 3, 4)

    def update_vertices(self, part: int, vertices: np.ndarray) -> None:
        v = np.ascontiguousarray(vertices, np.float32)
        if load().or_world_update_vertices(self.h, part, _p(v), v.shape[0]) != 0:
            raise ValueError("bad vertex update")

    def trace_instanced(self, rays: np.ndarray, any_hit: bool = False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        inst = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        bary = np.empty((n, 2), np.float32)
        load().or_trace_inst(self.h, _p(rays), n, 1 if any_hit else 0, _p(prim), _p(inst), _p(t), _p(bary))
        return prim, inst, t, bary


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
        if which == BUF_CACHE_QUERIES:
            return raw.view(np.uint32).reshape(-1, 8)
        if which == BUF_CACHE_TRAIN:
            return raw.view(np.uint32).reshape(-1, 12)
        return raw.view(np.uint32)

    def set_cache(self, enabled: bool, train_samples: int = 65536, cache: "OracleCache | None" = None):
        rc = load().or_renderer_set_cache(self.h, int(enabled), train_samples, cache.h if cache else None)
        if rc:
            raise ValueError("the radiance cache runs in corrected mode only")
        self._cache = cache   # keep the cache alive while the renderer uses it

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


# ---- learned radiance cache (nrc.cpp) ----
# XrCacheSample / OrCacheSample: pos[3] normal[3] wo[3] albedo[3] roughness kind target[3] pixel (72 B)
CACHE_SAMPLE_DTYPE = np.dtype([("pos", "<f4", 3), ("normal", "<f4", 3), ("wo", "<f4", 3), ("albedo", "<f4", 3),
                               ("roughness", "<f4"), ("kind", "<u4"), ("target", "<f4", 3), ("pixel", "<u4")])
NRC_MLP, NRC_GRID, NRC_MLP_GRAD, NRC_GRID_GRAD, NRC_MLP_M, NRC_MLP_V, NRC_GRID_M, NRC_GRID_V = range(8)


def pack_cache_samples(samples: np.ndarray) -> np.ndarray:
    s = np.ascontiguousarray(samples, CACHE_SAMPLE_DTYPE)
    rec = np.empty((len(s), 8), np.uint32)
    load().or_nrc_pack(_p(s.view(np.uint8)), len(s), _p(rec))
    return rec


class OracleCache:
    """CPU restatement of the learned radiance cache (hash grid + MLP + Adam)."""

    def __init__(self, seed: int = 1):
        self.h = load().or_nrc_create(seed)

    def set_bounds(self, lo, inv_extent: float):
        lo = np.ascontiguousarray(lo, np.float32)
        load().or_nrc_set_bounds(self.h, _p(lo), float(inv_extent))

    def param(self, which: int) -> np.ndarray:
        """A live view of one parameter / gradient / moment array."""
        n = C.c_size_t()
        ptr = load().or_nrc_params(self.h, which, C.byref(n))
        return np.ctypeslib.as_array(ptr, shape=(n.value,))

    def inputs(self, records: np.ndarray, exact: bool = False) -> np.ndarray:
        r = np.ascontiguousarray(records, np.uint32)
        x = np.empty((len(r), 64), np.float32)
        load().or_nrc_inputs(self.h, _p(r), len(r), _p(x), int(exact))
        return x

    def infer(self, records: np.ndarray, exact: bool = False) -> np.ndarray:
        r = np.ascontiguousarray(records, np.uint32)
        out = np.empty((len(r), 3), np.float32)
        load().or_nrc_infer(self.h, _p(r), len(r), _p(out), int(exact))
        return out

    def backward(self, records, targets, exact: bool = False, loss_kind: int = 0) -> float:
        r = np.ascontiguousarray(records, np.uint32)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 3)
        return load().or_nrc_backward(self.h, _p(r), _p(t), len(r), int(exact), loss_kind)

    def loss(self, records, targets, exact: bool = False, loss_kind: int = 0) -> float:
        r = np.ascontiguousarray(records, np.uint32)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 3)
        return load().or_nrc_loss(self.h, _p(r), _p(t), len(r), int(exact), loss_kind)

    def adam(self, lr, b1, b2, eps, bc1, bc2):
        load().or_nrc_adam(self.h, lr, b1, b2, eps, bc1, bc2)

    def close(self):
        if self.h:
            load().or_nrc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
