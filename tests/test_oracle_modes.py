"""Reference-mode behaviour and corrected-mode sanity of the oracle (CPU only)."""
import numpy as np

import xvk_ray_gb300 as xr
from oracle import binding as ob
from tests.helpers import camera_sequence


def _render(params, frames, bounces, scene=None):
    scene = scene or xr.Scene.cornell()
    r = ob.OracleRenderer(ob.OracleScene.from_scene(scene), params)
    for u in camera_sequence(scene, params.width, params.height, frames, bounces):
        r.render(u)
    return r


def test_reference_mode_marks_lights_white_and_misses_black():
    """ReSTIRGISpatialReuse.rgen.hlsl:80-89: n_view == 0 -> black, n_sample == 0 -> white."""
    W = H = 48
    scene = xr.Scene.cornell()
    scene.camera.fov_deg = 80.0                 # wide enough to see past the open front
    r = _render(xr.params_reference(W, H, write_hdr=1), 2, 4, scene)
    s = r.read(ob.BUF_SAMPLES).view(np.float32)
    hdr = r.read(ob.BUF_HDR)
    n_view = np.linalg.norm(s[:, 4:7], axis=1)
    n_sample = np.linalg.norm(s[:, 12:15], axis=1)
    light = (n_view > 0) & (n_sample == 0)
    miss = n_view == 0
    assert light.any() and miss.any()
    assert np.all(hdr[light, :3] == 1.0) and np.all(hdr[miss, :3] == 0.0)


def test_reference_mode_is_deterministic_and_finite():
    W = H = 32
    a = _render(xr.params_reference(W, H), 3, 10)
    b = _render(xr.params_reference(W, H), 3, 10)
    for buf in (ob.BUF_SAMPLES, ob.BUF_TEMPORAL, ob.BUF_SPATIAL):
        assert np.array_equal(a.read(buf), b.read(buf))
    assert np.all(np.isfinite(a.read(ob.BUF_HDR)))


def test_corrected_mode_converges_towards_the_fp64_reference():
    """ReSTIR GI lowers the error of the 1-spp estimate against a converged reference."""
    W = H = 32
    scene = xr.Scene.cornell()
    osc = ob.OracleScene.from_scene(scene)
    ubo0 = camera_sequence(scene, W, H, 1, 4)[0]
    ref = ob.pt_reference(osc, xr.params_default(W, H), ubo0, 1000, 1024)
    r = ob.OracleRenderer(osc, xr.params_default(W, H, write_pt=1))
    err_restir, err_pt = [], []
    for f, u in enumerate(camera_sequence(scene, W, H, 12, 4)):
        r.render(u)
        if f >= 6:
            hdr = r.read(ob.BUF_HDR)[:, :3].astype(np.float64)
            pt = r.read(ob.BUF_PT)[:, :3].astype(np.float64)
            err_restir.append(np.mean((hdr - ref) ** 2 / (ref ** 2 + 1e-2)))
            err_pt.append(np.mean((pt - ref) ** 2 / (ref ** 2 + 1e-2)))
    assert np.mean(err_restir) < 0.5 * np.mean(err_pt)
    assert abs(r.read(ob.BUF_PT)[:, :3].mean() / ref.mean() - 1) < 0.25
