"""Several scenes and views in one context (xr_upload_scenes / xr_set_views /
xr_render_views): every view is bit-identical to rendering it alone; frames
replayed from CUDA graphs and frames after the autotuner's launch choice are
bit-identical to direct launches."""
import numpy as np
import pytest

import xvk_ray_gb300 as xr
from xvk_ray_gb300 import _lib as L
from tests.helpers import camera_sequence

pytestmark = pytest.mark.gpu


def _scenes():
    return [xr.Scene.cornell(), xr.Scene.procedural(seed=3, n_objects=256, n_lights=8, extent=8.0)]


def _move(dz, dyaw):
    def f(frame, cam):
        cam.position[2] += dz
        cam.yaw_deg += dyaw
    return f


VIEWS = [(0, 64, 48), (1, 96, 64), (0, 40, 40), (1, 33, 17)]
MOVES = [_move(-0.01, 0.2), _move(-0.01, 0.3), _move(0.02, -0.4), _move(0.0, 0.5)]


def _sequences(scenes, frames, bounces=4):
    return [camera_sequence(scenes[s], w, h, frames, bounces, move=MOVES[k]) for k, (s, w, h) in enumerate(VIEWS)]


def _alone(scene, view, seq, params_fn):
    _, w, h = view
    with xr.Renderer(w, h) as r:
        r.set_params(params_fn(w, h, write_hdr=1))
        r.upload_scene(scene)
        r.build_bvh()
        for u in seq:
            r.render(u)
        return r.read_output(L.XR_OUT_HDR)


def _batch(scenes, seqs, params_fn, frames, graphs=False, tuning=None):
    r = xr.Renderer(8, 8)
    r.upload_scenes(scenes)
    r.set_views(VIEWS, params_fn(8, 8, write_hdr=1))
    if graphs:
        r.set_graphs(True)
    if tuning is not None:
        if isinstance(tuning, dict):
            r.set_tuning(**tuning)
        else:
            r.set_tuning(tuning=tuning) if hasattr(tuning, "refill_min") else r.set_tuning(*tuning)
    for f in range(frames):
        r.render_views([seqs[v][f] for v in range(len(VIEWS))])
    out = [r.read_view_output(v, L.XR_OUT_HDR) for v in range(len(VIEWS))]
    st = r.stats()
    r.close()
    return out, st


@pytest.mark.parametrize("mode", ["corrected", "reference"])
def test_views_match_single_renders(mode):
    params_fn = xr.params_default if mode == "corrected" else xr.params_reference
    scenes = _scenes() if mode == "corrected" else [xr.Scene.cornell(), xr.Scene.cornell()]
    frames = 3
    seqs = _sequences(scenes, frames)
    got, st = _batch(scenes, seqs, params_fn, frames)
    assert st.error_flags == 0
    for k, view in enumerate(VIEWS):
        ref = _alone(scenes[view[0]], view, seqs[k], params_fn)
        assert np.array_equal(got[k].view(np.uint32), ref.view(np.uint32)), (mode, k)


def test_graph_replay_matches_direct_launches():
    scenes = _scenes()
    frames = 5
    seqs = _sequences(scenes, frames)
    direct, _ = _batch(scenes, seqs, xr.params_default, frames, graphs=False)
    graphed, st = _batch(scenes, seqs, xr.params_default, frames, graphs=True)
    assert st.frames == frames
    for k in range(len(VIEWS)):
        assert np.array_equal(direct[k].view(np.uint32), graphed[k].view(np.uint32)), k


def test_autotuned_launches_do_not_change_results():
    scenes = _scenes()
    frames = 3
    seqs = _sequences(scenes, frames)
    plain, _ = _batch(scenes, seqs, xr.params_default, frames)
    with xr.Renderer(8, 8) as r:
        r.upload_scenes(scenes)
        r.set_views(VIEWS, xr.params_default(8, 8, write_hdr=1))
        t = r.autotune([[seqs[v][f] for v in range(len(VIEWS))] for f in range(frames)])
    assert t.configs_tried >= 15 and 0 < t.ms_per_frame <= t.ms_default
    # the tuner's choice, fewer persistent CTAs, and every tile / queue knob away from its default
    knobs = dict(refill_min=4, postpone_below=16, ray_bundle=2, temporal_block=256, spatial_block=64)
    for tuning in (t, (3, 1), knobs, dict(ray_bundle=1, temporal_block=32, spatial_block=256, refill_min=12)):
        tuned, _ = _batch(scenes, seqs, xr.params_default, frames, tuning=tuning)
        for k in range(len(VIEWS)):
            assert np.array_equal(plain[k].view(np.uint32), tuned[k].view(np.uint32)), (tuning, k)


def test_view_of_an_empty_scene_renders_misses():
    base = xr.Scene.cornell()
    empty = xr.Scene(base.vertices, base.indices[:0].copy(), base.materials, base.ranges, base.camera)
    scenes = [empty, base]
    views = [(0, 16, 16), (1, 16, 16)]
    with xr.Renderer(8, 8) as r:
        r.upload_scenes(scenes)
        r.set_views(views, xr.params_default(8, 8, write_hdr=1))
        seq = camera_sequence(base, 16, 16, 1, 4)[0]
        r.render_views([seq, seq])
        e = r.read_view_output(0, L.XR_OUT_HDR)
        c = r.read_view_output(1, L.XR_OUT_HDR)
        assert r.stats().error_flags == 0
    assert np.all(e[:, :3] == 0.0)
    assert c[:, :3].max() > 0.0
