"""The CUDA kernels in reference mode against the reference's own shader source.

The expected values in tests/golden/ref_passes.npz and ref_frames.npz were
computed by shader/HLSL/ReSTIRGI/*.hlsl themselves (compiled as C++ by
oracle/refpin, tests/golden/make_ref_fixtures.py).  Through the C ABI the
kernels must reproduce every field the reference-mode layout keeps -- the
samples, the temporal and spatial reservoirs (both ping-pong halves) -- bit for
bit up to the sign of a zero (tests.helpers.canon), and the RGBA8 image within
one step (the gamma is each side's powf).
"""
import json

import numpy as np
import pytest

import xvk_ray_gb300 as xr
from tests.helpers import RES_FIELDS, SAMPLE_FIELDS, canon
from tests.helpers import RES_INT_WORDS, SAMPLE_INT_WORDS, field_digests
from tests.test_refpin import frame_scene, frame_sequences, load_fixture

pytestmark = pytest.mark.gpu
XR = xr._lib

GPU_SAMPLE_FIELDS = {k: SAMPLE_FIELDS[k] for k in ("x_view", "materialID", "n_view", "randSeed", "x_sample", "p_q",
                                                   "n_sample", "L_out", "f")}


@pytest.mark.parametrize("name", frame_sequences())
def test_frames_match_reference_source(name):
    g = load_fixture("ref_frames.npz")
    meta = json.loads(str(g[f"{name}_meta"]))
    scene = frame_scene(g, meta["scene"], name)
    W, H = meta["width"], meta["height"]
    digests = json.loads(str(g[f"{name}_digests"]))
    with xr.Renderer(W, H) as r:
        r.set_params(xr.params_reference(W, H))
        r.upload_scene(scene)
        r.build_bvh()
        for f, (ub, want) in enumerate(zip(g[f"{name}_ubos"], digests)):
            r.render(XR.XrUniformBufferObject.from_buffer_copy(ub.tobytes()))
            got = {"samples." + k: v for k, v in field_digests(r.read_buffer(XR.XR_BUF_SAMPLES), GPU_SAMPLE_FIELDS,
                                                                SAMPLE_INT_WORDS).items()}
            for which, label in ((XR.XR_BUF_TEMPORAL, "temporal"), (XR.XR_BUF_SPATIAL, "spatial")):
                got.update({f"{label}.{k}": v for k, v in field_digests(r.read_buffer(which), RES_FIELDS,
                                                                         RES_INT_WORDS).items()})
            bad = sorted(k for k in got if got[k] != want[k])
            assert not bad, f"frame {f}: {bad}"
            ldr = r.read_output(XR.XR_OUT_LDR8).reshape(-1, 4)[:, :3].astype(np.int32)
            diff = np.abs(ldr - g[f"{name}_ldr"][f][:, :3].astype(np.int32))
            assert diff.max() <= 1, f"frame {f}: image"


@pytest.mark.parametrize("case", ["kat", "surface"])
def test_fixed_candidate_passes_match_reference_source(case):
    g = load_fixture("ref_passes.npz")
    W, H = int(g[f"{case}_width"]), int(g[f"{case}_height"])
    ubo = XR.XrUniformBufferObject.from_buffer_copy(g[f"{case}_ubo"].tobytes())

    def same(a, b, label):
        for k, sl in RES_FIELDS.items():
            assert np.array_equal(canon(a, RES_INT_WORDS)[:, sl], canon(b, RES_INT_WORDS)[:, sl]), f"{label}.{k}"

    with xr.Renderer(W, H) as r:
        r.set_params(xr.params_reference(W, H))
        r.upload_scene(xr.Scene.cornell())
        r.build_bvh()
        r.write_buffer(XR.XR_BUF_SAMPLES, g[f"{case}_samples"])
        r.write_buffer(XR.XR_BUF_TEMPORAL, g[f"{case}_temporal_in"])
        ubo.reuse = 0
        r.run_pass(ubo, 1)
        same(r.read_buffer(XR.XR_BUF_TEMPORAL), g[f"{case}_temporal_out"], "temporal")
        same(r.read_buffer(XR.XR_BUF_SPATIAL), g[f"{case}_spatial_after_temporal"], "spatial after temporal")
        for reuse in (1, 0):
            ubo.reuse = reuse
            r.run_pass(ubo, 2)
            same(r.read_buffer(XR.XR_BUF_SPATIAL), g[f"{case}_spatial_out_reuse{reuse}"], f"spatial reuse={reuse}")
            ldr = r.read_output(XR.XR_OUT_LDR8).reshape(-1, 4)[:, :3].astype(np.int32)
            assert np.abs(ldr - g[f"{case}_ldr_reuse{reuse}"][:, :3].astype(np.int32)).max() <= 1
