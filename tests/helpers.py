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
