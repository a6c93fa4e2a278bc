"""Generates the golden vectors under tests/golden/ (run from the repo root).

  rng_kat.json        random.hlsl:1-20 -- InitRandomSeed and the first NextRandom /
                      RandomFloat outputs for a set of pixels and frames
  temporal_kat.npz    ReSTIRGITemporalReuse.rgen.hlsl (reference behaviour) on an 8x8
                      image of handcrafted candidates and previous reservoirs

Both come from tests/pyref.py, a pure-Python restatement written independently
of the C++ oracle; the oracle and the CUDA path are checked against them.
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from tests import pyref  # noqa: E402

HERE = Path(__file__).resolve().parent


def rng_kat():
    cases = []
    for (x, y, w, frame) in [(0, 0, 1920, 0), (1, 0, 1920, 0), (0, 1, 1920, 0), (1919, 1079, 1920, 9999),
                             (37, 11, 256, 3), (255, 255, 256, 7), (640, 360, 1280, 123), (5, 5, 7, 4294967294)]:
        s = pyref.init_random_seed(x, y, w, frame)
        st, u32, f32 = s, [], []
        for _ in range(8):
            st, r = pyref.next_random(st)
            u32.append(r)
        st = s
        for _ in range(8):
            st, f = pyref.random_float(st)
            f32.append(int(np.float32(f).view(np.uint32)))
        cases.append({"x": x, "y": y, "width": w, "frame": frame, "seed": s, "next_random": u32,
                      "random_float_bits": f32})
    (HERE / "rng_kat.json").write_text(json.dumps({"source": "random.hlsl:1-20", "cases": cases}, indent=1))


def temporal_kat():
    import xvk_ray_gb300 as xr

    W = H = 8
    n = W * H
    rng = np.random.default_rng(20261203)
    cam = xr._lib.XrCamera((0.0, 1.0, 3.4), 0.0, 0.0, 45.0)
    u0 = xr.camera_ubo(cam, W, H, None, 0, 4)
    cam.position[0] = 0.05
    cam.yaw_deg = 1.5
    ubo = xr.camera_ubo(cam, W, H, u0, 5, 4, reuse=False)
    samples = np.zeros((n, 24), np.uint32)
    # f of a Lambertian visible point is albedo / pi of its material (BSDF.hlsl:22-24)
    albedo = xr.Scene.cornell().materials[:, :3]
    inv_pi = np.float32(1.0 / 3.14159265359)
    for p in range(n):
        s = pyref.init_sample()
        kind = rng.integers(0, 10)
        if kind == 0:                      # miss at the visible point
            samples[p] = pyref.sample_words(s)
            continue
        s["x_view"] = rng.uniform([-1, 0, -1], [1, 2, 1]).astype(np.float32)
        s["n_view"] = pyref.normalize(rng.normal(size=3).astype(np.float32))
        if kind == 1:                      # light seen directly: n_sample stays zero
            samples[p] = pyref.sample_words(s)
            continue
        s["materialID"] = int(rng.integers(0, 3))
        s["randSeed"] = int(rng.integers(0, 2**32))
        s["x_sample"] = rng.uniform([-1, 0, -1], [1, 2, 1]).astype(np.float32)
        s["n_sample"] = pyref.normalize(rng.normal(size=3).astype(np.float32))
        s["p_q"] = np.float32(0.0 if kind == 2 else rng.uniform(0.01, 0.32))
        s["L_out"] = (np.zeros(3) if kind == 3 else rng.uniform(0, 5, size=3)).astype(np.float32)
        s["f"] = (albedo[s["materialID"]] * inv_pi).astype(np.float32)
        samples[p] = pyref.sample_words(s)
    temporal = np.zeros((2 * n, 28), np.uint32)
    for i in range(2 * n):
        r = pyref.init_reservoir()
        if rng.integers(0, 4):
            r["W"] = np.float32(rng.uniform(0, 3))
            r["w_sum"] = np.float32(rng.uniform(0, 10))
            r["m"] = int(rng.integers(0, 40))
            s = pyref.sample_fields(samples[rng.integers(0, n)])
            s["x_sample"] = rng.uniform([-1, 0, -1], [1, 2, 1]).astype(np.float32)
            s["L_out"] = rng.uniform(0, 4, size=3).astype(np.float32)
            r["s"] = s
        temporal[i] = pyref.reservoir_words(r)
    spatial = np.zeros((2 * n, 28), np.uint32)
    ubo_dict = {"current_frame": ubo.current_frame, "view_prev": np.array(ubo.view_prev, np.float32),
                "projection_prev": np.array(ubo.projection_prev, np.float32)}
    t_out, s_out = pyref.temporal_reference_mode(samples.copy(), temporal.copy(), spatial.copy(), ubo_dict, W, H)
    np.savez_compressed(HERE / "temporal_kat.npz", width=W, height=H, ubo=np.frombuffer(xr.ubo_bytes(ubo), np.uint8),
                        samples=samples, temporal_in=temporal, spatial_in=spatial, temporal_out=t_out, spatial_out=s_out)


if __name__ == "__main__":
    rng_kat()
    temporal_kat()
    print("golden vectors written to", HERE)
