"""Reservoir passes of the CUDA path on fixed candidates.

The golden candidates of tests/golden/temporal_kat.npz (restated in pure Python
by tests/pyref.py) go through the C ABI (xr_write_buffer + xr_run_pass) and
must come back bit for bit; the spatial pass is then compared with the oracle
on the same inputs, and randomised candidates exercise both modes.
"""
from pathlib import Path

import numpy as np
import pytest

import xvk_ray_gb300 as xr
from oracle import binding as ob
from tests.helpers import RES_FIELDS, diff_words

pytestmark = pytest.mark.gpu
XR = xr._lib
GOLDEN = Path(__file__).resolve().parent / "golden"


def _gpu(params, scene):
    r = xr.Renderer(params.width, params.height)
    r.set_params(params)
    r.upload_scene(scene)
    r.build_bvh()
    return r


def test_temporal_pass_on_golden_candidates():
    kat = np.load(GOLDEN / "temporal_kat.npz")
    W, H = int(kat["width"]), int(kat["height"])
    ubo = XR.XrUniformBufferObject.from_buffer_copy(kat["ubo"].tobytes())
    scene = xr.Scene.cornell()
    with _gpu(xr.params_reference(W, H, write_hdr=1), scene) as r:
        r.write_buffer(XR.XR_BUF_SAMPLES, kat["samples"])
        r.write_buffer(XR.XR_BUF_TEMPORAL, kat["temporal_in"])
        r.run_pass(ubo, 1)
        gt = r.read_buffer(XR.XR_BUF_TEMPORAL)
        gs = r.read_buffer(XR.XR_BUF_SPATIAL)
        for k in ("w_sum", "W", "m", "x_sample", "n_sample", "L_out", "f"):
            assert diff_words(gt, kat["temporal_out"], RES_FIELDS[k]) == 0, k
            assert diff_words(gs, kat["spatial_out"], RES_FIELDS[k]) == 0, k
        # spatial pass on the same inputs against the oracle
        o = ob.OracleRenderer(ob.OracleScene.from_scene(scene), xr.params_reference(W, H))
        o.set_samples(kat["samples"], ubo)
        o.write_temporal(kat["temporal_in"])
        o.run_pass(ubo, 1)
        ubo.reuse = 1
        o.run_pass(ubo, 2)
        r.run_pass(ubo, 2)
        gsp, osp = r.read_buffer(XR.XR_BUF_SPATIAL), o.read(ob.BUF_SPATIAL)
        for k in ("w_sum", "W", "m", "x_sample", "n_sample", "L_out", "f"):
            assert diff_words(gsp, osp, RES_FIELDS[k]) == 0, k
        written = o.read(ob.BUF_WRITTEN).astype(bool)
        gh, oh = r.read_output(XR.XR_OUT_HDR), o.read(ob.BUF_HDR)
        assert np.array_equal(gh[written].view(np.uint32), oh[written].view(np.uint32))


def test_corrected_mode_passes_on_frame_candidates():
    """Candidates of a rendered frame re-run through the oracle's passes alone."""
    from tests.helpers import camera_sequence

    scene = xr.Scene.procedural(seed=8, n_objects=128, n_lights=6, extent=6.0)
    W, H = 96, 64
    p = xr.params_default(W, H, write_hdr=1)
    ubos = camera_sequence(scene, W, H, 3, 4)
    with _gpu(p, scene) as r:
        o = ob.OracleRenderer(ob.OracleScene.from_scene(scene), p)
        r.render(ubos[0])
        r.render(ubos[1])
        s1 = r.read_buffer(XR.XR_BUF_SAMPLES)
        t1 = r.read_buffer(XR.XR_BUF_TEMPORAL)
        r.render(ubos[2])
        s2 = r.read_buffer(XR.XR_BUF_SAMPLES)
        o.set_samples(s1, ubos[1])
        o.end_frame()                      # frame 1's G-buffer becomes "previous"
        o.write_temporal(t1)
        o.set_samples(s2, ubos[2])
        o.run_pass(ubos[2], 1)
        o.run_pass(ubos[2], 2)
        gt, ot = r.read_buffer(XR.XR_BUF_TEMPORAL), o.read(ob.BUF_TEMPORAL)
        gs, os_ = r.read_buffer(XR.XR_BUF_SPATIAL), o.read(ob.BUF_SPATIAL)[: W * H]
        for k in ("W", "m", "x_sample", "L_out"):
            assert diff_words(gt, ot, RES_FIELDS[k]) == 0, k
            assert diff_words(gs, os_, RES_FIELDS[k]) == 0, k
        # pixels whose primary ray found a surface (the others show emission the
        # candidate buffers do not carry)
        valid = s2[:, 3] != 0xFFFFFFFF
        gh, oh = r.read_output(XR.XR_OUT_HDR), o.read(ob.BUF_HDR)
        assert np.array_equal(gh[valid].view(np.uint32), oh[valid].view(np.uint32))
