"""Shared helpers of the parity tests."""
from __future__ import annotations

import numpy as np

import xvk_ray_gb300 as xr
from oracle import binding as ob

SAMPLE_FIELDS = {           # word ranges of ReSTIRGISample (ReSTIRGICommon.hlsl:6-20)
    "x_view": slice(0, 3), "materialID": slice(3, 4), "n_view": slice(4, 7), "randSeed": slice(7, 8),
    "x_sample": slice(8, 11), "p_q": slice(11, 12), "n_sample": slice(12, 15), "pad1": slice(15, 16),
    "L_out": slice(16, 19), "f": slice(20, 23),
}
RES_FIELDS = {              # word ranges of ReSTIRGIReservoir (ReSTIRGICommon.hlsl:22-30)
    "w_sum": slice(0, 1), "W": slice(1, 2), "m": slice(2, 3),
    "x_sample": slice(12, 15), "n_sample": slice(16, 19), "L_out": slice(20, 23), "f": slice(24, 27),
}
# the reservoir's copy of the rest of its sample (ReSTIRGIReservoir.s)
RES_SAMPLE_FIELDS = {"s.x_view": slice(4, 7), "s.materialID": slice(7, 8), "s.n_view": slice(8, 11),
                     "s.randSeed": slice(11, 12), "s.p_q": slice(15, 16)}
SAMPLE_INT_WORDS = [3, 7, 15, 19, 23]                        # materialID, randSeed, pad1..pad3
RES_INT_WORDS = [2, 3] + [4 + w for w in SAMPLE_INT_WORDS]   # m, pad, the sample's integer words


def canon(words: np.ndarray, int_words) -> np.ndarray:
    """Record words with every float -0.0 turned into +0.0 (integer words as they
    are).  The reference maps normals through its identity instance transform,
    whose products with zeros make the sign of a zero the driver's choice; every
    other bit is compared."""
    w = np.array(words, np.uint32, copy=True)
    neg0 = w == 0x80000000
    neg0[:, list(int_words)] = False
    w[neg0] = 0
    return w


def canon_floats(a: np.ndarray) -> np.ndarray:
    """Float array bits with -0.0 as +0.0."""
    w = np.array(a, np.float32, copy=True).view(np.uint32)
    w[w == 0x80000000] = 0
    return w


def field_digests(words: np.ndarray, fields: dict, int_words) -> dict:
    """SHA-1 of each field's canonical words (see canon)."""
    import hashlib
    c = canon(words, int_words)
    return {k: hashlib.sha1(np.ascontiguousarray(c[:, sl]).tobytes()).hexdigest() for k, sl in fields.items()}


def unorm8(v: np.ndarray) -> np.ndarray:
    """An RGBA8 UNORM store of float colours: clamp to [0, 1], * 255 + 0.5, truncate
    (float32 arithmetic, the oracle's and the kernels' conversion)."""
    v = np.clip(np.asarray(v, np.float32), np.float32(0), np.float32(1))
    return (v * np.float32(255.0) + np.float32(0.5)).astype(np.int32).astype(np.uint8)


def random_rays(rng: np.random.Generator, n: int, lo, hi, tmin=1e-4, tmax=1e4) -> np.ndarray:
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = tmin
    rays[:, 4:7] = d.astype(np.float32)
    rays[:, 7] = tmax
    return rays


def camera_sequence(scene, w, h, frames, bounces, move=None, sky=False, reuse=True):
    """UBOs of a scripted camera path (move(frame, cam) edits an XrCamera)."""
    cam = xr._lib.XrCamera.from_buffer_copy(scene.camera)
    prev = None
    out = []
    for f in range(frames):
        if move is not None:
            move(f, cam)
        u = xr.camera_ubo(cam, w, h, prev, f, bounces, sky=sky, reuse=reuse)
        prev = u
        out.append(u)
    return out


def diff_words(a: np.ndarray, b: np.ndarray, cols: slice) -> int:
    """Number of rows whose words in `cols` differ bit-wise."""
    return int(np.sum(np.any(a[:, cols] != b[:, cols], axis=1)))


def box_scene(rng: np.random.Generator, n_boxes: int, extent: float, step: float = 1.0 / 16.0,
              light: bool = True) -> "xr.Scene":
    """Axis-aligned boxes (and an emissive quad above them) whose coordinates are
    multiples of `step`: translating the scene by multiples of `step` is exact in
    float, so instanced and baked copies trace bit-identically."""
    verts, idx, mats = [], [], []
    mats.append([0.7, 0.6, 0.5, 1.0, 0.0, 0.0, 0.0, 0.0])     # Lambertian
    mats.append([0.3, 0.5, 0.8, 1.0, 0.0, 0.4, 0.0, 0.0])     # Lambertian, other colour
    # corner k has x = hi if bit 0 is set, y if bit 1, z if bit 2
    faces = [((0, 2, 6, 4), (-1, 0, 0)), ((1, 3, 7, 5), (1, 0, 0)), ((0, 1, 5, 4), (0, -1, 0)),
             ((2, 6, 7, 3), (0, 1, 0)), ((0, 1, 3, 2), (0, 0, -1)), ((4, 6, 7, 5), (0, 0, 1))]

    def q(v):
        return np.round(np.asarray(v, np.float64) / step) * step

    def add_quad(p4, n, m):
        base = len(verts)
        for p in p4:
            verts.append([p[0], p[1], p[2], n[0], n[1], n[2], 0.0, 0.0, 0.0])
            verts[-1][8] = np.array([m], np.int32).view(np.float32)[0]
        idx.extend([base, base + 1, base + 2, base, base + 2, base + 3])

    for b in range(n_boxes):
        c = q(rng.uniform(-extent, extent, 3))
        h = q(rng.uniform(0.25, 1.0, 3) * extent / 4.0) + step
        lo, hi = c - h, c + h
        corners = [[(hi if (k >> a) & 1 else lo)[a] for a in range(3)] for k in range(8)]
        for f, n in faces:
            add_quad([corners[i] for i in f], n, b % 2)
    if light:
        mats.append([4.0, 4.0, 4.0, 1.0, 0.0, 0.0, 0.0, 0.0])
        mats[-1][7] = np.array([3], np.uint32).view(np.float32)[0]   # DiffuseLight
        y = extent * 1.5
        s = q(extent / 3.0)
        add_quad([[-s, y, -s], [-s, y, s], [s, y, s], [s, y, -s]], (0, -1, 0), len(mats) - 1)
    m = np.array(mats, np.float32)
    m[:, 4] = np.array([-1] * m.shape[0], np.int32).view(np.float32)   # no base-colour texture
    v = np.array(verts, np.float32)
    cam = xr._lib.XrCamera()
    cam.position[:] = [0.0, 0.0, extent * 3.0]
    cam.yaw_deg, cam.pitch_deg, cam.fov_deg = 0.0, 0.0, 60.0
    return xr.Scene(v, np.array(idx, np.uint32), m, np.zeros((1, 2), np.uint32), cam)


def rotation(axis, deg: float) -> np.ndarray:
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    t = np.radians(deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * K @ K


def affine(R, t) -> np.ndarray:
    """3x4 object-to-world matrix [R | t] (float32 values)."""
    m = np.zeros((3, 4), np.float64)
    m[:, :3] = R
    m[:, 3] = t
    return m.astype(np.float32)


def bake_instances(scenes, instances) -> "tuple[xr.Scene, np.ndarray, np.ndarray]":
    """One flat scene holding every instance's triangles in world space (float64
    transform, rounded to float).  Also returns, per baked primitive, its instance
    and its primitive in the concatenation of `scenes`."""
    verts, idx, mats, inst_of, prim_of = [], [], [], [], []
    prim0 = np.cumsum([0] + [s.n_triangles for s in scenes])
    mat0 = np.cumsum([0] + [s.materials.shape[0] for s in scenes])
    for s in scenes:
        mats.append(s.materials)
    nv = 0
    for i, (k, m) in enumerate(instances):
        s = scenes[k]
        m = np.asarray(m, np.float64).reshape(3, 4)
        v = s.vertices.copy()
        p = s.vertices[:, 0:3].astype(np.float64)
        v[:, 0:3] = (p @ m[:, :3].T + m[:, 3]).astype(np.float32)
        n = s.vertices[:, 3:6].astype(np.float64) @ np.linalg.inv(m[:, :3])
        v[:, 3:6] = (n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)).astype(np.float32)
        mi = s.vertices[:, 8].view(np.int32).copy()
        mi[mi >= 0] += int(mat0[k])
        v[:, 8] = mi.view(np.float32)
        verts.append(v)
        idx.append(s.global_indices() + nv)
        nv += v.shape[0]
        inst_of.append(np.full(s.n_triangles, i, np.int32))
        prim_of.append(np.arange(s.n_triangles, dtype=np.int32) + int(prim0[k]))
    sc = xr.Scene(np.concatenate(verts), np.concatenate(idx).astype(np.uint32), np.concatenate(mats),
                  np.zeros((1, 2), np.uint32), scenes[0].camera)
    return sc, np.concatenate(inst_of), np.concatenate(prim_of)


def scene_digest(sc) -> str:
    """SHA-1 of a scene's arrays and textures."""
    import hashlib
    h = hashlib.sha1()
    for a in (sc.vertices, sc.indices, sc.materials, sc.ranges):
        h.update(np.ascontiguousarray(a).tobytes())
    for t in sc.textures:
        h.update(np.ascontiguousarray(t).tobytes())
    return h.hexdigest()
