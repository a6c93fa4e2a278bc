"""Pure-Python restatement of parts of the reference shaders (test infrastructure).

An implementation independent of the C++ oracle, used to pin it:
  random.hlsl:1-20                              (InitRandomSeed, NextRandom, RandomFloat)
  ReSTIRGICommon.hlsl:43-73                     (InitReservoir, UpdateReservoir, MergeReservoir)
  ReSTIRGITemporalReuse.rgen.hlsl:33-131        (temporal reuse, reference behaviour)
  Sampling.hlsl:39-56                           (WorldToScreenUV)
All float arithmetic is numpy float32 scalars, one rounding per operation in
the order of the shader source; integers wrap at 32 bits.
"""
from __future__ import annotations

import numpy as np

F = np.float32
M32 = 0xFFFFFFFF


# ---- random.hlsl ----
def init_random_seed(x: int, y: int, width: int, frame: int) -> int:
    s = (x * 1 + y * width) & M32
    s = (s ^ 61) ^ (s >> 16)
    s = (s * 9) & M32
    s = s ^ (s >> 4)
    s = (s * 0x27D4EB2D) & M32
    s = s ^ (s >> 15)
    return (s * (frame + 1)) & M32


def next_random(state: int) -> tuple[int, int]:
    state = (state * 747796405 + 2891336453) & M32
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & M32
    return state, (word >> 22) ^ word


def random_float(state: int) -> tuple[int, np.float32]:
    state, r = next_random(state)
    return state, F(r & 0x00FFFFFF) / F(16777216.0)


# ---- float3 helpers ----
def v3(a) -> np.ndarray:
    return np.asarray(a, dtype=np.float32).reshape(3)


def dot(a, b) -> np.float32:
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def length(a) -> np.float32:
    return np.sqrt(dot(a, a))


def normalize(a) -> np.ndarray:
    r = F(1.0) / np.sqrt(dot(a, a))
    return np.array([a[0] * r, a[1] * r, a[2] * r], np.float32)


def mat_mul(m: np.ndarray, v) -> np.ndarray:
    """HLSL mul(M, v) with a column-major float[16], summed left to right."""
    o = np.zeros(4, np.float32)
    for r in range(4):
        o[r] = m[0 + r] * v[0] + m[4 + r] * v[1] + m[8 + r] * v[2] + m[12 + r] * v[3]
    return o


def world_to_screen_uv(p, view, proj):
    vp = mat_mul(view, [p[0], p[1], p[2], F(1.0)])
    cp = mat_mul(proj, vp)
    nx, ny = cp[0] / cp[3], cp[1] / cp[3]
    return nx * F(0.5) + F(0.5), ny * F(0.5) + F(0.5)


# ---- ReSTIRGISample / ReSTIRGIReservoir as word arrays (24 / 28 uint32) ----
def sample_fields(w: np.ndarray) -> dict:
    f = w.view(np.float32)
    return {"x_view": f[0:3].copy(), "materialID": int(w[3]), "n_view": f[4:7].copy(), "randSeed": int(w[7]),
            "x_sample": f[8:11].copy(), "p_q": f[11], "n_sample": f[12:15].copy(), "L_out": f[16:19].copy(),
            "f": f[20:23].copy()}


def sample_words(s: dict) -> np.ndarray:
    w = np.zeros(24, np.uint32)
    f = w.view(np.float32)
    f[0:3] = s["x_view"]; w[3] = s["materialID"]; f[4:7] = s["n_view"]; w[7] = s["randSeed"]
    f[8:11] = s["x_sample"]; f[11] = s["p_q"]; f[12:15] = s["n_sample"]; f[16:19] = s["L_out"]; f[20:23] = s["f"]
    return w


def init_sample() -> dict:
    z = np.zeros(3, np.float32)
    return {"x_view": z.copy(), "materialID": M32, "n_view": z.copy(), "randSeed": 0, "x_sample": z.copy(),
            "p_q": F(0.0), "n_sample": z.copy(), "L_out": z.copy(), "f": z.copy()}


def init_reservoir() -> dict:
    return {"w_sum": F(0.0), "W": F(0.0), "m": 0, "s": init_sample()}


def reservoir_words(r: dict) -> np.ndarray:
    w = np.zeros(28, np.uint32)
    f = w.view(np.float32)
    f[0] = r["w_sum"]; f[1] = r["W"]; w[2] = r["m"] & M32
    w[4:28] = sample_words(r["s"])
    return w


def reservoir_fields(w: np.ndarray) -> dict:
    f = w.view(np.float32)
    return {"w_sum": f[0], "W": f[1], "m": int(w[2]), "s": sample_fields(w[4:28])}


def update_reservoir(r: dict, s: dict, w_new, state: int) -> int:
    r["w_sum"] = r["w_sum"] + w_new
    r["m"] = (r["m"] + 1) & M32
    state, u = random_float(state)
    if u < w_new / max(F(1e-10), r["w_sum"]):
        r["s"] = dict(s)
    return state


def merge_reservoir(t: dict, src: dict, p_hat, state: int) -> int:
    m0 = t["m"]
    w_new = p_hat * src["W"] * F(src["m"])
    state = update_reservoir(t, src["s"], w_new, state)
    t["m"] = (m0 + src["m"]) & M32
    return state


def eval_target(s: dict, x_curr, n_curr) -> np.float32:
    wi = normalize(s["x_sample"] - x_curr)
    c = dot(n_curr, wi)
    if c <= F(0.0):
        return F(0.0)
    return length(s["L_out"])


def temporal_reference_mode(samples: np.ndarray, temporal: np.ndarray, spatial: np.ndarray, ubo: dict,
                            width: int, height: int, m_max: int = 30):
    """ReSTIRGITemporalReuse.rgen.hlsl:41-131 over all pixels; the previous G-buffer is the
    current one (the reference's aliasing) and the motion vector goes through RG16F.
    Mutates and returns (temporal, spatial) word arrays of 2N reservoirs."""
    n = width * height
    frame = ubo["current_frame"]
    pp = frame % 2
    cur, prev = pp * n, (1 - pp) * n
    valid = samples[:, 3] != M32
    for p in range(n):
        x, y = p % width, p // width
        s = sample_fields(samples[p])
        if length(s["n_sample"]) == F(0.0):
            temporal[cur + p] = reservoir_words(init_reservoir())
            spatial[cur + p] = reservoir_words(init_reservoir())
            continue
        cu = ((F(x) + F(0.5)) / F(width), (F(y) + F(0.5)) / F(height))
        pu = world_to_screen_uv(s["x_view"], ubo["view_prev"], ubo["projection_prev"])
        mv = (F(np.float16(cu[0] - pu[0])), F(np.float16(cu[1] - pu[1])))
        fx = (cu[0] - mv[0]) * F(width)
        fy = (cu[1] - mv[1]) * F(height)
        found = False
        r_prev = None
        if F(-1.0) < fx < F(width) and F(-1.0) < fy < F(height):
            q = int(fy) * width + int(fx)
            if valid[q]:
                r_prev = reservoir_fields(temporal[prev + q].copy())
                found = True
            else:
                spatial[cur + p] = reservoir_words(init_reservoir())
        state = init_random_seed(x, y, width, frame)
        x_curr = s["x_view"]
        n_curr = normalize(s["n_view"])
        r = init_reservoir()
        tp = eval_target(s, x_curr, n_curr)
        w_new = tp / s["p_q"] if s["p_q"] > F(1e-6) else F(0.0)
        state = update_reservoir(r, s, w_new, state)
        if found:
            state = merge_reservoir(r, r_prev, eval_target(r_prev["s"], x_curr, n_curr), state)
        else:
            r["m"] = 1
        if r["m"] > m_max:
            r["w_sum"] = r["w_sum"] * (F(m_max) / F(r["m"]))
            r["m"] = m_max
        tpf = eval_target(r["s"], x_curr, n_curr)
        r["W"] = r["w_sum"] / (F(r["m"]) * tpf) if (tpf > F(1e-6) and r["m"] > 0) else F(0.0)
        temporal[cur + p] = reservoir_words(r)
    return temporal, spatial
