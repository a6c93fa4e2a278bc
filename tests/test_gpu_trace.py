"""Hit-id parity of the GPU LBVH/CWBVH traversal against the oracle's brute force / BVH.

Reference semantics: TraceRay with opaque triangles, no culling, TMin/TMax
(ReSTIRGIInitialSample.rgen.hlsl:76-98); ties broken by the lowest primitive id.
"""
import numpy as np
import pytest

import xvk_ray_gb300 as xr
from oracle import binding as ob
from tests.helpers import random_rays

pytestmark = pytest.mark.gpu


def _renderer_for(scene, w=8, h=8):
    r = xr.Renderer(w, h)
    r.set_params(xr.params_default(w, h))
    r.upload_scene(scene)
    r.build_bvh()
    return r


@pytest.mark.parametrize("any_hit", [False, True])
def test_cornell_hits_bit_exact(any_hit):
    scene = xr.Scene.cornell()
    rng = np.random.default_rng(7)
    rays = random_rays(rng, 200000, [-1.2, -0.2, -1.2], [1.2, 2.2, 1.6])
    with _renderer_for(scene) as r:
        gp, gt, gb = r.trace(rays, any_hit)
    osc = ob.OracleScene.from_scene(scene)
    op, ot, obary = osc.trace(rays, any_hit)
    if any_hit:
        assert np.array_equal(gp >= 0, op >= 0)
    else:
        assert np.array_equal(gp, op)
        hit = op >= 0
        assert np.array_equal(gt[hit].view(np.uint32), ot[hit].view(np.uint32))
        assert np.array_equal(gb[hit].view(np.uint32), obary[hit].view(np.uint32))


def test_axis_aligned_and_edge_rays():
    """Rays along the axes and through shared edges/vertices of the Cornell quads."""
    scene = xr.Scene.cornell()
    v = scene.vertices[:, :3]
    rng = np.random.default_rng(3)
    targets = np.concatenate([v, (v[scene.indices[0::3]] + v[scene.indices[1::3]]) * 0.5]).astype(np.float32)
    origins = np.array([[0.0, 1.0, 3.0], [0.0, 1.0, 0.0], [0.3, 0.5, 0.2]], np.float32)
    rays = []
    for o in origins:
        d = targets - o
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        r = np.zeros((len(d), 8), np.float32)
        r[:, :3] = o; r[:, 3] = 1e-4; r[:, 4:7] = d; r[:, 7] = 1e4
        rays.append(r)
    axes = np.eye(3, dtype=np.float32)
    for s in (1.0, -1.0):
        for a in axes:
            r = np.zeros((64, 8), np.float32)
            r[:, :3] = rng.uniform(-0.9, 0.9, size=(64, 3)) + np.array([0, 1.0, 0])
            r[:, 3] = 0.0; r[:, 4:7] = s * a; r[:, 7] = 1e4
            rays.append(r)
    rays = np.concatenate(rays)
    with _renderer_for(scene) as r:
        gp, gt, _ = r.trace(rays)
    op, ot, _ = ob.OracleScene.from_scene(scene).trace(rays)
    assert np.array_equal(gp, op)
    assert np.array_equal(gt[op >= 0].view(np.uint32), ot[op >= 0].view(np.uint32))


@pytest.mark.parametrize("builder", ["ploc", "lbvh"])
@pytest.mark.parametrize("n_objects", [64, 2048])
def test_procedural_hits_bit_exact(n_objects, builder, monkeypatch):
    monkeypatch.setenv("XR_BVH_BUILDER", builder)
    scene = xr.Scene.procedural(seed=5, n_objects=n_objects, extent=10.0)
    rng = np.random.default_rng(11)
    rays = random_rays(rng, 100000, [-12, 0.0, -12], [12, 4.0, 12])
    with _renderer_for(scene) as r:
        gp, gt, gb = r.trace(rays)
        ga, _, _ = r.trace(rays, any_hit=True)
        st = r.stats()
    osc = ob.OracleScene.from_scene(scene)
    op, ot, obary = osc.trace(rays)
    assert st.error_flags == 0
    assert st.bvh_triangles >= scene.n_triangles   # slots: large triangles are split into pieces
    assert np.array_equal(gp, op)
    hit = op >= 0
    assert np.array_equal(gt[hit].view(np.uint32), ot[hit].view(np.uint32))
    assert np.array_equal(gb[hit].view(np.uint32), obary[hit].view(np.uint32))
    assert np.array_equal(ga >= 0, hit)


def test_degenerate_scenes():
    """0, 1 and 2 triangles, and a zero-area triangle."""
    base = xr.Scene.cornell()
    rng = np.random.default_rng(1)
    rays = random_rays(rng, 5000, [-1, 0, -1], [1, 2, 1])
    for ntri in (0, 1, 2, 3):
        s = xr.Scene(base.vertices, base.indices[: 3 * ntri].copy(), base.materials, base.ranges, base.camera)
        with _renderer_for(s) as r:
            gp, gt, _ = r.trace(rays)
        if ntri:
            op, ot, _ = ob.OracleScene.from_scene(s).trace(rays)
            assert np.array_equal(gp, op)
        else:
            assert np.all(gp == -1)
    v = base.vertices.copy()
    v[base.indices[2], :3] = v[base.indices[1], :3]     # collapse triangle 0 to a segment
    s = xr.Scene(v, base.indices, base.materials, base.ranges, base.camera)
    with _renderer_for(s) as r:
        gp, _, _ = r.trace(rays)
    op, _, _ = ob.OracleScene.from_scene(s).trace(rays)
    assert np.array_equal(gp, op)


@pytest.mark.parametrize("any_hit", [False, True])
def test_axis_aligned_rays_bounded_work(any_hit):
    """Directions with exactly zero components (+0 and -0) keep their box tests.

    A zero component has an infinite reciprocal; the traversal must still cull
    on that axis rather than walk the whole tree.  Hits match the oracle and the
    node visits per ray stay a small fraction of the node count.
    """
    scene = xr.Scene.procedural(seed=5, n_objects=2048, extent=10.0)
    rng = np.random.default_rng(17)
    n = 4096
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0] = rng.uniform(-11, 11, n); rays[:, 1] = rng.uniform(0.001, 3.0, n); rays[:, 2] = rng.uniform(-11, 11, n)
    rays[:, 3] = 1e-4
    axis = rng.integers(0, 3, n)
    sign = np.where(rng.integers(0, 2, n) == 0, 1.0, -1.0).astype(np.float32)
    zero = np.where(rng.integers(0, 2, (n, 3)) == 0, np.float32(0.0), np.float32(-0.0))
    rays[:, 4:7] = zero
    rays[np.arange(n), 4 + axis] = sign
    rays[:, 7] = 1e4
    with _renderer_for(scene) as r:
        gp, gt, _ = r.trace(rays, any_hit)
        st = r.stats()
    op, ot, _ = ob.OracleScene.from_scene(scene).trace(rays, any_hit)
    assert st.error_flags == 0
    if any_hit:
        assert np.array_equal(gp >= 0, op >= 0)
    else:
        assert np.array_equal(gp, op)
        assert np.array_equal(gt[op >= 0].view(np.uint32), ot[op >= 0].view(np.uint32))
    assert st.query_rays == n
    assert st.query_node_visits / n < 0.02 * st.bvh_nodes
