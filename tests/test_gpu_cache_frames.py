"""Frames with the learned radiance cache: records bit-exact against the oracle,
candidates within the tolerance of the BF16 network, training every frame, and
what the trained cache gains over plain ReSTIR GI (relMSE against the FP64
reference of the plain path tracer)."""
import numpy as np
import pytest

import xvk_ray_gb300 as xr
from xvk_ray_gb300 import _lib as L
from oracle import binding as ob
from tests.helpers import SAMPLE_FIELDS, camera_sequence

pytestmark = pytest.mark.gpu

L_OUT_TOL = 5e-3     # relative norm error of the cache radiance in the candidates


def _cache_params(train_samples, enabled=1):
    cp = xr.cache_params_default()
    cp.enabled = enabled
    cp.train_samples = train_samples
    return cp


def _by_pixel(rec):
    return rec[np.argsort(rec[:, 3], kind="stable")]


def test_cache_frames_match_oracle():
    scene = xr.Scene.procedural(seed=3, n_objects=256, n_lights=8, extent=8.0)
    W, H = 96, 64

    def move(f, cam):
        cam.position[2] -= 0.01
        cam.yaw_deg += 0.2

    p = xr.params_default(W, H, write_hdr=1, write_pt=1)
    ubos = camera_sequence(scene, W, H, 3, 4, move=move)
    train_n = 1024
    with xr.Renderer(W, H) as r:
        r.set_params(p)
        r.upload_scene(scene)
        r.build_bvh()
        r.cache.set_params(_cache_params(train_n))
        r.cache.reset(2)
        st = r.cache.stats()
        oc = ob.OracleCache(2)
        oc.set_bounds(np.array(st.bounds_lo, np.float32), st.inv_extent)
        o = ob.OracleRenderer(ob.OracleScene.from_scene(scene), p)
        o.set_cache(True, train_n, oc)
        for f, u in enumerate(ubos):
            # the oracle predicts with the weights the frame starts from
            oc.param(ob.NRC_MLP)[:] = r.cache.read(L.XR_CACHE_MLP)
            oc.param(ob.NRC_GRID)[:] = r.cache.read(L.XR_CACHE_GRID)
            r.render(u)
            o.render(u)
            gq, oq = _by_pixel(r.cache.read(L.XR_CACHE_QUERIES)), o.read(ob.BUF_CACHE_QUERIES)
            gt, ot = _by_pixel(r.cache.read(L.XR_CACHE_TRAIN_RECORDS)), o.read(ob.BUF_CACHE_TRAIN)
            assert len(oq) > 500 and len(ot) > 20, (f, len(oq), len(ot))
            assert np.array_equal(gq, oq), f
            assert np.array_equal(gt, ot), f
            cs = r.cache.stats()
            assert cs.queries == len(oq) and cs.train_samples == len(ot)
            assert cs.steps == f + 1 and np.isfinite(cs.loss)
            gs, os_ = r.read_buffer(L.XR_BUF_SAMPLES), o.read(ob.BUF_SAMPLES)
            lo = SAMPLE_FIELDS["L_out"]
            other = np.ones(24, bool)
            other[lo] = False
            assert np.array_equal(gs[:, other], os_[:, other]), f
            gl, ol = gs[:, lo].view(np.float32), os_[:, lo].view(np.float32)
            qpix = oq[:, 3]
            rest = np.setdiff1d(np.arange(W * H), qpix)
            assert np.array_equal(gl[rest], ol[rest]), f
            err = np.linalg.norm(gl[qpix] - ol[qpix]) / np.linalg.norm(ol[qpix])
            assert err < L_OUT_TOL, (f, err)


def test_cache_disabled_frames_unchanged():
    """The cache off (parameters set, enabled = 0) leaves the plain pipeline bit-identical."""
    scene = xr.Scene.cornell()
    W, H = 64, 48
    p = xr.params_default(W, H, write_hdr=1)
    ubos = camera_sequence(scene, W, H, 2, 4)
    out = []
    for use in (False, True):
        with xr.Renderer(W, H) as r:
            r.set_params(p)
            r.upload_scene(scene)
            r.build_bvh()
            if use:
                r.cache.set_params(_cache_params(4096, enabled=0))
            for u in ubos:
                r.render(u)
            out.append(r.read_output(L.XR_OUT_HDR))
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


def test_reference_mode_rejects_cache():
    scene = xr.Scene.cornell()
    W, H = 32, 32
    with xr.Renderer(W, H) as r:
        r.set_params(xr.params_reference(W, H))
        r.upload_scene(scene)
        r.build_bvh()
        r.cache.set_params(_cache_params(256))
        with pytest.raises(xr.XrError):
            r.render(camera_sequence(scene, W, H, 1, 4)[0])


def test_cache_frames_replayed_from_graphs():
    """Training and inference inside replayed frame graphs.  With a learning rate
    of 1e-30 every update is below half an ulp of the FP32 weights (and the FP16 /
    BF16 inference images round it away), so graph replay and direct launches must give
    bit-identical images and records (one Adam step counted per frame either way).
    With the default rate the float-order nondeterminism of the gradient atomics
    makes the two trajectories drift apart, so the check is on the size of the
    updates: bias correction advanced on the device gives the same mean weight
    change as the host-driven path (a stuck correction would roughly double it)."""
    scene = xr.Scene.procedural(seed=3, n_objects=256, n_lights=8, extent=8.0)
    W, H = 96, 64
    ubos = camera_sequence(scene, W, H, 6, 4)

    def run(graphs, lr):
        with xr.Renderer(W, H) as r:
            r.set_params(xr.params_default(W, H, write_hdr=1))
            r.upload_scene(scene)
            r.build_bvh()
            cp = _cache_params(1024)
            cp.learning_rate = lr
            r.cache.set_params(cp)
            r.cache.reset(2)
            w0 = r.cache.read(L.XR_CACHE_MLP)
            r.set_graphs(graphs)
            for u in ubos:
                r.render(u)
            cs = r.cache.stats()
            assert cs.steps == len(ubos) and np.isfinite(cs.loss) and cs.train_samples > 0
            return (r.read_output(L.XR_OUT_HDR)[:, :3].copy(), r.cache.read(L.XR_CACHE_QUERIES),
                    r.cache.read(L.XR_CACHE_MLP) - w0)

    img_d, q_d, _ = run(False, 1e-30)
    img_g, q_g, _ = run(True, 1e-30)
    assert np.array_equal(img_d.view(np.uint32), img_g.view(np.uint32))
    assert np.array_equal(_by_pixel(q_d), _by_pixel(q_g))   # appended in warp order: compare by pixel

    _, _, dw_d = run(False, 1e-2)
    _, _, dw_g = run(True, 1e-2)
    step_d, step_g = np.abs(dw_d).mean(), np.abs(dw_g).mean()
    assert step_d > 1e-4
    assert 0.9 < step_g / step_d < 1.1, (step_g, step_d)


def _relmse(img, ref):
    x = img[:, :3].astype(np.float64)
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))


def test_trained_cache_lowers_relmse():
    """What the trained network gains over the method without it: the Cornell box
    (128 x 128, static camera, path depth 8), 64 frames of ReSTIR GI with and
    without the learned cache (training every frame), relMSE of the last 16
    frames against the FP64-accumulated plain path tracer (1024 spp).  Measured on
    GB300: 0.43x of plain ReSTIR GI (0.52x at depth 4); the test asks for < 0.7x.
    It also checks that the adaptive training selection yields about
    train_samples records a frame."""
    scene = xr.Scene.cornell()
    W = H = 128
    ubos = camera_sequence(scene, W, H, 64, 8)
    rel = {}
    for cache in (False, True):
        with xr.Renderer(W, H) as r:
            r.set_params(xr.params_default(W, H, write_hdr=1, write_pt=1))
            r.upload_scene(scene)
            r.build_bvh()
            if cache:
                r.cache.set_params(_cache_params(2048))
                r.cache.reset(3)
            ref = r.render_reference(ubos[0], 1_000_000, 1024)
            vals = []
            for f, u in enumerate(ubos):
                r.render(u)
                if f >= 48:
                    vals.append(_relmse(r.read_output(L.XR_OUT_HDR), ref))
                if cache and f >= 4:
                    n = r.cache.stats().train_samples
                    assert 1500 < n < 2600, (f, n)
            rel[cache] = float(np.mean(vals))
    assert rel[True] < 0.7 * rel[False], rel
