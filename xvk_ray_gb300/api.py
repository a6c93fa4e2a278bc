"""Python view of the C ABI: scenes as numpy arrays, a Renderer per context.

Every call goes through libxr.so; numpy holds host arrays only.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None and a.size else 0


@dataclass
class Scene:
    """Flat scene arrays in the reference's upload layout (src/Asset/Scene.cpp:16-49).

    vertices: (nv, 9) float32 -- pos3, normal3, uv2, material index (int32 bits)
    indices:  (ni,)  uint32, relative to the owning range's vertex offset
    materials: (nm, 8) float32 -- base colour4, texture index (int32 bits),
               fuzziness, refraction index, model (uint32 bits)
    ranges:   (nr, 2) uint32 -- (index offset, vertex offset) per model
    """
    vertices: np.ndarray
    indices: np.ndarray
    materials: np.ndarray
    ranges: np.ndarray
    camera: L.XrCamera
    textures: list = field(default_factory=list)   # (height, width, 4) uint8 RGBA, row 0 = v 0

    @property
    def n_triangles(self) -> int:
        return int(self.indices.size // 3)

    def global_indices(self) -> np.ndarray:
        """Absolute vertex index per index slot (each range's vertex offset applied)."""
        out = self.indices.astype(np.uint32).copy()
        offs = list(self.ranges[:, 0]) + [self.indices.size]
        for r in range(self.ranges.shape[0]):
            out[offs[r]:offs[r + 1]] += self.ranges[r, 1]
        return out

    def save(self, path) -> None:
        """Writes the scene (arrays, camera, RGBA8 textures) to one .npz file, e.g. to
        keep a glTF scene in the upload layout and skip parsing it again."""
        tex = {f"texture{i}": t for i, t in enumerate(self.textures)}
        np.savez_compressed(path, vertices=self.vertices, indices=self.indices, materials=self.materials,
                            ranges=self.ranges, camera=np.frombuffer(bytes(self.camera), np.uint8),
                            n_textures=len(self.textures), **tex)

    @staticmethod
    def load(path) -> "Scene":
        """A scene written by Scene.save."""
        with np.load(path) as z:
            cam = L.XrCamera.from_buffer_copy(z["camera"].tobytes())
            tex = [np.ascontiguousarray(z[f"texture{i}"]) for i in range(int(z["n_textures"]))]
            return Scene(np.ascontiguousarray(z["vertices"]), np.ascontiguousarray(z["indices"]),
                         np.ascontiguousarray(z["materials"]), np.ascontiguousarray(z["ranges"]), cam, tex)

    @staticmethod
    def _generate(fn, *args) -> "Scene":
        lib = L.load()
        d = L.XrSceneData()
        L.check(fn(*args, C.byref(d)))
        v = np.zeros((d.vertex_count, 9), np.float32)
        i = np.zeros(d.index_count, np.uint32)
        m = np.zeros((d.material_count, 8), np.float32)
        d.vertices, d.indices, d.materials = _ptr(v), _ptr(i), _ptr(m)
        L.check(fn(*args, C.byref(d)))
        cam = L.XrCamera()
        C.memmove(C.byref(cam), C.byref(d.camera), C.sizeof(cam))
        return Scene(v, i, m, np.zeros((1, 2), np.uint32), cam)

    @staticmethod
    def cornell() -> "Scene":
        return Scene._generate(L.load().xr_scene_cornell)

    @staticmethod
    def procedural(seed: int = 1, n_objects: int = 4096, n_lights: int = 16, extent: float = 40.0,
                   sphere_subdiv: int = 2) -> "Scene":
        desc = L.XrProceduralDesc(seed, n_objects, n_lights, extent, sphere_subdiv)
        lib = L.load()
        return Scene._generate(lib.xr_scene_procedural, C.byref(desc))


def params_default(width: int, height: int, **kw) -> L.XrParams:
    p = L.XrParams()
    L.load().xr_params_default(C.byref(p), width, height)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def params_reference(width: int, height: int, **kw) -> L.XrParams:
    p = L.XrParams()
    L.load().xr_params_reference(C.byref(p), width, height)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def camera_ubo(cam: L.XrCamera, width: int, height: int, prev: L.XrUniformBufferObject | None, frame: int,
               bounces: int, sky: bool = False, reuse: bool = True) -> L.XrUniformBufferObject:
    """PathTracer::GetUniformBufferObject (src/pathTracer.cpp:169-201)."""
    out = L.XrUniformBufferObject()
    L.check(L.load().xr_camera_ubo(C.byref(cam), width, height, C.byref(prev) if prev is not None else None, frame,
                                   bounces, 1 if sky else 0, 1 if reuse else 0, C.byref(out)))
    return out


def ubo_bytes(u: L.XrUniformBufferObject) -> bytes:
    return C.string_at(C.addressof(u), C.sizeof(u))


class Renderer:
    """One libxr context (one GPU, one stream)."""

    def __init__(self, width: int, height: int, device: int = 0):
        lib = L.load()
        self._lib = lib
        h = C.c_void_p()
        L.check(lib.xr_create(C.byref(L.XrDeviceDesc(device, width, height)), C.byref(h)))
        self.ctx = h
        self.width, self.height = width, height
        self.cache = Cache(self)
        self._pending_reads = []    # the arrays asynchronous image reads copy into, oldest first

    def _c(self, status: int) -> None:
        L.check(status, self.ctx)

    def close(self) -> None:
        if self.ctx:
            self._lib.xr_destroy(self.ctx)   # finishes a pending image read first
            self.ctx = None
        self._pending_reads = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- scene / BVH --
    def upload_textures(self, textures: "list[np.ndarray]") -> None:
        """RGBA8 textures, each (height, width, 4) uint8 with row 0 at v = 0."""
        keep = [np.ascontiguousarray(t, np.uint8) for t in textures]
        arr = (L.XrTexture * max(len(keep), 1))()
        for k, t in enumerate(keep):
            arr[k].width, arr[k].height = t.shape[1], t.shape[0]
            arr[k].rgba8 = C.cast(_ptr(t), C.POINTER(C.c_uint8))
        self._c(self._lib.xr_upload_textures(self.ctx, C.cast(arr, C.c_void_p), len(keep)))

    def upload_scene(self, scene: Scene) -> None:
        if scene.textures:
            self.upload_textures(scene.textures)
        v = np.ascontiguousarray(scene.vertices, np.float32)
        i = np.ascontiguousarray(scene.indices, np.uint32)
        m = np.ascontiguousarray(scene.materials, np.float32)
        r = np.ascontiguousarray(scene.ranges, np.uint32)
        self._c(self._lib.xr_upload_scene(self.ctx, _ptr(v), v.shape[0], _ptr(i), i.size, _ptr(m), m.shape[0],
                                          _ptr(r), r.shape[0]))

    def build_bvh(self) -> None:
        self._c(self._lib.xr_build_bvh(self.ctx))

    def set_params(self, p: L.XrParams) -> None:
        self._c(self._lib.xr_set_params(self.ctx, C.byref(p)))
        self.width, self.height = p.width, p.height

    # -- frames --
    # -- several scenes / views in one context --
    def upload_scenes(self, scenes: "list[Scene]") -> None:
        """Uploads the scenes and builds their BVHs (views then pick them by index)."""
        keep = []
        arr = (L.XrSceneData * len(scenes))()
        for k, sc in enumerate(scenes):
            v = np.ascontiguousarray(sc.vertices, np.float32)
            i = np.ascontiguousarray(sc.global_indices(), np.uint32)
            m = np.ascontiguousarray(sc.materials, np.float32)
            keep += [v, i, m]
            arr[k].vertices, arr[k].vertex_count = _ptr(v), v.shape[0]
            arr[k].indices, arr[k].index_count = _ptr(i), i.size
            arr[k].materials, arr[k].material_count = _ptr(m), m.shape[0]
        self._c(self._lib.xr_upload_scenes(self.ctx, C.cast(arr, C.c_void_p), len(scenes)))

    def set_views(self, views: "list[tuple[int, int, int]]", params: L.XrParams) -> None:
        """views: (scene index, width, height) per view; params are shared (their extent is ignored)."""
        arr = (L.XrView * len(views))(*[L.XrView(*v) for v in views])
        self.views = list(views)
        self._c(self._lib.xr_set_views(self.ctx, C.cast(arr, C.c_void_p), len(views), C.byref(params)))

    def render_views(self, ubos: "list[L.XrUniformBufferObject]") -> None:
        arr = (L.XrUniformBufferObject * len(ubos))(*ubos)
        self._c(self._lib.xr_render_views(self.ctx, C.cast(arr, C.c_void_p)))

    def read_view_output(self, view: int, which: int = L.XR_OUT_LDR8) -> np.ndarray:
        _, w, h = self.views[view]
        if which == L.XR_OUT_LDR8:
            out = np.empty((w * h, 4), np.uint8)
        else:
            out = np.empty((w * h, 4), np.float32)
        self._c(self._lib.xr_read_view_output(self.ctx, view, which, _ptr(out), out.nbytes))
        return out

    def render_reference_views(self, ubos: "list[L.XrUniformBufferObject]", frame0: int, spp: int) -> "list[np.ndarray]":
        """FP64 reference of every view (list of (W*H, 3) float64 arrays)."""
        arr = (L.XrUniformBufferObject * len(ubos))(*ubos)
        n = sum(w * h for _, w, h in self.views)
        out = np.empty((n, 3), np.float64)
        self._c(self._lib.xr_render_reference_views(self.ctx, C.cast(arr, C.c_void_p), frame0, spp, _ptr(out)))
        res, off = [], 0
        for _, w, h in self.views:
            res.append(out[off:off + w * h])
            off += w * h
        return res

    def set_graphs(self, enabled: bool) -> None:
        self._c(self._lib.xr_set_graphs(self.ctx, 1 if enabled else 0))

    def autotune(self, frames: "list[list[L.XrUniformBufferObject]]") -> L.XrTuning:
        """frames: per frame, the UBO of every view (or a single UBO for a one-view context)."""
        flat = [u for f in frames for u in (f if isinstance(f, (list, tuple)) else [f])]
        arr = (L.XrUniformBufferObject * len(flat))(*flat)
        t = L.XrTuning()
        self._c(self._lib.xr_autotune(self.ctx, C.cast(arr, C.c_void_p), len(frames), C.byref(t)))
        return t

    def set_tuning(self, trace_ctas_per_sm: int = 0, shade_ctas_per_sm: int = 0, *, refill_min: int = 0,
                   postpone_below: int = 0, ray_bundle: int = 0, temporal_block: int = 0, spatial_block: int = 0,
                   tuning: "L.XrTuning | None" = None) -> None:
        """A launch configuration (0 = the default of each knob), or one xr_autotune chose."""
        t = tuning if tuning is not None else L.XrTuning(trace_ctas_per_sm, shade_ctas_per_sm, 0.0, 0.0, 0, refill_min,
                                                         postpone_below, ray_bundle, temporal_block, spatial_block)
        self._c(self._lib.xr_set_tuning(self.ctx, C.byref(t)))

    def render(self, ubo: L.XrUniformBufferObject) -> None:
        self._c(self._lib.xr_render_frame(self.ctx, C.byref(ubo)))

    def sync(self) -> None:
        self._c(self._lib.xr_sync(self.ctx))

    def read_output(self, which: int = L.XR_OUT_LDR8, out: np.ndarray | None = None) -> np.ndarray:
        n = self.width * self.height
        if out is None:
            out = np.empty((n, 4), np.uint8 if which == L.XR_OUT_LDR8 else np.float32)
        self._c(self._lib.xr_read_output(self.ctx, which, _ptr(out), out.nbytes))
        return out

    def render_reference(self, ubo: L.XrUniformBufferObject, frame0: int, spp: int) -> np.ndarray:
        """FP64-accumulated plain path tracer over `spp` samples: (width*height, 3) float64."""
        out = np.empty((self.width * self.height, 3), np.float64)
        self._c(self._lib.xr_render_reference(self.ctx, C.byref(ubo), frame0, spp, _ptr(out)))
        return out

    def read_output_async(self, out: np.ndarray) -> None:
        """Starts copying the last frame's RGBA8 image into `out` (width*height*4
        bytes, preferably page-locked: PinnedBuffer.array) and returns at once; the
        image is there after the wait_output() that covers it (reads are waited for
        oldest first; at most two in flight).  `out` is kept alive until then."""
        if out.nbytes < self.width * self.height * 4 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("read_output_async: need a contiguous array of width*height*4 bytes")
        self._c(self._lib.xr_read_output_async(self.ctx, _ptr(out), out.nbytes))
        self._pending_reads.append(out)

    def wait_output(self) -> None:
        """Blocks until the oldest read_output_async() copy not yet waited for has landed."""
        self._c(self._lib.xr_wait_output(self.ctx))
        if self._pending_reads:
            self._pending_reads.pop(0)

    def output_device_ptr(self, which: int = L.XR_OUT_LDR8) -> int:
        p = C.c_void_p()
        self._c(self._lib.xr_output_device_ptr(self.ctx, which, C.byref(p)))
        return p.value

    def stats(self) -> L.XrStats:
        s = L.XrStats()
        self._c(self._lib.xr_get_stats(self.ctx, C.byref(s)))
        return s

    # -- parity access in the reference layouts --
    def read_buffer(self, which: int) -> np.ndarray:
        n = C.c_size_t()
        self._c(self._lib.xr_read_buffer(self.ctx, which, None, 0, C.byref(n)))
        words = 24 if which == L.XR_BUF_SAMPLES else 28
        out = np.empty(n.value // 4, np.uint32)
        self._c(self._lib.xr_read_buffer(self.ctx, which, _ptr(out), out.nbytes, None))
        return out.reshape(-1, words)

    def write_buffer(self, which: int, words: np.ndarray) -> None:
        w = np.ascontiguousarray(words, np.uint32)
        self._c(self._lib.xr_write_buffer(self.ctx, which, _ptr(w), w.nbytes))

    def run_pass(self, ubo: L.XrUniformBufferObject, pass_id: int) -> None:
        self._c(self._lib.xr_run_pass(self.ctx, C.byref(ubo), pass_id))

    def trace(self, rays: np.ndarray, any_hit: bool = False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        bary = np.empty((n, 2), np.float32)
        self._c(self._lib.xr_trace_rays(self.ctx, _ptr(rays), n, 1 if any_hit else 0, _ptr(prim), _ptr(t),
                                        _ptr(bary)))
        return prim, t, bary

    def trace_instanced(self, rays: np.ndarray, any_hit: bool = False):
        """trace() that also returns each hit's instance (-1: miss or no instances)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        inst = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        bary = np.empty((n, 2), np.float32)
        self._c(self._lib.xr_trace_rays_instanced(self.ctx, _ptr(rays), n, 1 if any_hit else 0, _ptr(prim),
                                                  _ptr(inst), _ptr(t), _ptr(bary)))
        return prim, inst, t, bary

    def set_instances(self, instances) -> None:
        """instances: (scene index, 3x4 object-to-world matrix) pairs, or an array of
        INSTANCE_DTYPE records (no per-instance Python work); [] clears them."""
        arr = pack_instances(instances)
        self._c(self._lib.xr_set_instances(self.ctx, arr.ctypes.data_as(C.c_void_p), arr.shape[0]))

    def instance_transforms(self, n: int) -> np.ndarray:
        """(n, 2, 3, 4): object-to-world and world-to-object of the first n instances."""
        out = np.empty((n, 24), np.float32)
        self._c(self._lib.xr_get_instance_transforms(self.ctx, _ptr(out), n))
        return out.reshape(n, 2, 3, 4)

    def update_vertices(self, scene: int, vertices: np.ndarray) -> None:
        """New vertices (same count and layout as uploaded) of a scene, then a refit of its BVH."""
        v = np.ascontiguousarray(vertices, np.float32)
        self._c(self._lib.xr_update_vertices(self.ctx, int(scene), _ptr(v), v.shape[0]))


# host layout of XrInstance (56 B)
INSTANCE_DTYPE = np.dtype([("scene", "<u4"), ("reserved", "<u4"), ("object_to_world", "<f4", 12)])
assert INSTANCE_DTYPE.itemsize == C.sizeof(L.XrInstance)


def pack_instances(instances) -> np.ndarray:
    """XrInstance records of (scene index, 3x4 matrix) pairs; records pass through."""
    if isinstance(instances, np.ndarray) and instances.dtype == INSTANCE_DTYPE:
        return np.ascontiguousarray(instances)
    n = len(instances)
    arr = np.zeros(n, INSTANCE_DTYPE)
    if n:
        arr["scene"] = [int(s) for s, _ in instances]
        arr["object_to_world"] = np.asarray([np.asarray(m, np.float64).reshape(12) for _, m in instances],
                                            np.float64).astype(np.float32)
    return arr


# host layout of XrCacheSample (72 B)
CACHE_SAMPLE_DTYPE = np.dtype([("pos", "<f4", 3), ("normal", "<f4", 3), ("wo", "<f4", 3), ("albedo", "<f4", 3),
                               ("roughness", "<f4"), ("kind", "<u4"), ("target", "<f4", 3), ("pixel", "<u4")])
assert CACHE_SAMPLE_DTYPE.itemsize == C.sizeof(L.XrCacheSample)


def cache_params_default() -> L.XrCacheParams:
    p = L.XrCacheParams()
    L.load().xr_cache_params_default(C.byref(p))
    return p


class Cache:
    """The learned radiance cache of one Renderer (xr_cache_* entry points)."""

    ARRAY_FLOATS = {0: 17408, 1: 16 * (1 << 19) * 2}

    def __init__(self, renderer: "Renderer"):
        self._r = renderer

    def _c(self, status):
        self._r._c(status)

    @property
    def _ctx(self):
        return self._r.ctx

    def set_params(self, p: L.XrCacheParams) -> None:
        self._c(L.load().xr_cache_set_params(self._ctx, C.byref(p)))

    def params(self) -> L.XrCacheParams:
        p = L.XrCacheParams()
        self._c(L.load().xr_cache_get_params(self._ctx, C.byref(p)))
        return p

    def reset(self, seed: int = 1) -> None:
        self._c(L.load().xr_cache_reset(self._ctx, seed))

    def set_bounds(self, lo, inv_extent: float) -> None:
        lo = np.ascontiguousarray(lo, np.float32)
        self._c(L.load().xr_cache_set_bounds(self._ctx, _ptr(lo), float(inv_extent)))

    def query(self, samples: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(samples, CACHE_SAMPLE_DTYPE)
        out = np.empty((len(s), 3), np.float32)
        self._c(L.load().xr_cache_query(self._ctx, _ptr(s.view(np.uint8)), len(s), _ptr(out)))
        return out

    def train(self, samples: np.ndarray, apply: bool = True) -> float:
        s = np.ascontiguousarray(samples, CACHE_SAMPLE_DTYPE)
        loss = C.c_float()
        self._c(L.load().xr_cache_train(self._ctx, _ptr(s.view(np.uint8)), len(s), int(apply), C.byref(loss)))
        return loss.value

    def step(self) -> None:
        self._c(L.load().xr_cache_step(self._ctx))

    def read(self, which: int) -> np.ndarray:
        n = C.c_size_t()
        self._c(L.load().xr_cache_read(self._ctx, which, None, 0, C.byref(n)))
        if which in (L.XR_CACHE_QUERIES, L.XR_CACHE_TRAIN_RECORDS):
            out = np.empty(n.value // 4, np.uint32)
            if n.value:
                self._c(L.load().xr_cache_read(self._ctx, which, _ptr(out), out.nbytes, None))
            return out.reshape(-1, 8 if which == L.XR_CACHE_QUERIES else 12)
        out = np.empty(n.value // 4, np.uint32 if which == L.XR_CACHE_ADAM_STEP else np.float32)
        self._c(L.load().xr_cache_read(self._ctx, which, _ptr(out), out.nbytes, None))
        return out

    def write(self, which: int, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, np.uint32 if which == L.XR_CACHE_ADAM_STEP else np.float32)
        self._c(L.load().xr_cache_write(self._ctx, which, _ptr(v), v.nbytes))

    def checkpoint(self) -> dict:
        """The cache's whole trained state: arrays 0..7, the Adam step count and the
        hash encoding's bounds (the scene cube the positions are normalised to)."""
        state = {w: self.read(w).copy() for w in list(range(8)) + [L.XR_CACHE_ADAM_STEP]}
        st = self.stats()
        state["bounds"] = (tuple(float(v) for v in st.bounds_lo), float(st.inv_extent))
        return state

    def restore(self, state: dict) -> None:
        """Writes a checkpoint back.  The bounds are restored too, so a context with
        another scene (another scene cube) predicts as the checkpointed one did."""
        for w, v in state.items():
            if w == "bounds":
                continue
            self.write(w, v)
        if "bounds" in state:
            lo, inv = state["bounds"]
            self.set_bounds(lo, inv)

    def stats(self) -> L.XrCacheStats:
        st = L.XrCacheStats()
        self._c(L.load().xr_cache_get_stats(self._ctx, C.byref(st)))
        return st


class PinnedBuffer:
    """Page-locked host memory (cudaMallocHost) viewed as a numpy array."""

    def __init__(self, nbytes: int):
        p = C.c_void_p()
        L.check(L.load().xr_alloc_host(nbytes, C.byref(p)))
        self.ptr = p.value
        self.nbytes = nbytes
        self.array = np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(self.ptr))

    def free(self) -> None:
        if self.ptr:
            L.load().xr_free_host(self.ptr)
            self.ptr = None
