"""Instances in the oracle (CPU): the world-to-object inverse, identity and
translated instances against flat scenes (bit-exact), rotated and scaled
instances against a baked world (same hits up to the rounding of baking)."""
import numpy as np

import xvk_ray_gb300 as xr
from oracle import binding as ob
from tests.helpers import affine, bake_instances, box_scene, random_rays, rotation


def _mats():
    return [affine(np.eye(3), [0, 0, 0]),
            affine(rotation([0, 1, 0], 30) * 1.5, [2.0, -1.0, 0.5]),
            affine(rotation([1, 1, 0], -75) @ np.diag([0.5, 2.0, 1.0]), [-3.0, 0.25, 4.0])]


def test_world_to_object_is_the_inverse():
    world = ob.OracleWorld([ob.OracleScene.from_scene(xr.Scene.cornell())])
    mats = _mats()
    world.set_instances([(0, m) for m in mats])
    X = world.transforms()
    for k, m in enumerate(mats):
        assert np.array_equal(X[k, 0], m)
        A = np.vstack([m.astype(np.float64), [0, 0, 0, 1]])
        assert np.allclose(X[k, 1], np.linalg.inv(A)[:3], rtol=1e-6, atol=1e-6)


def test_singular_instance_is_rejected():
    world = ob.OracleWorld([ob.OracleScene.from_scene(xr.Scene.cornell())])
    m = affine(np.diag([1.0, 0.0, 1.0]), [0, 0, 0])
    try:
        world.set_instances([(0, m)])
    except ValueError:
        return
    raise AssertionError("a singular transform was accepted")


def test_identity_instance_traces_like_the_scene():
    scene = xr.Scene.procedural(seed=5, n_objects=96, n_lights=4, extent=6.0)
    flat = ob.OracleScene.from_scene(scene)
    world = ob.OracleWorld([flat])
    world.set_instances([(0, affine(np.eye(3), [0, 0, 0]))])
    rays = random_rays(np.random.default_rng(1), 20000, -6.0, 6.0)
    for any_hit in (False, True):
        p0, t0, b0 = flat.trace(rays, any_hit)
        p1, i1, t1, b1 = world.trace_instanced(rays, any_hit)
        assert np.array_equal(p0, p1)
        assert np.all(i1[p1 >= 0] == 0) and np.all(i1[p1 < 0] == -1)
        if not any_hit:
            assert np.array_equal(t0.view(np.uint32), t1.view(np.uint32))
            assert np.array_equal(b0.view(np.uint32), b1.view(np.uint32))


def test_translated_instances_trace_like_the_baked_scene():
    """Grid-aligned geometry, translations and ray origins: baking is exact, so the
    instanced world and the baked scene give bit-identical closest hits."""
    rng = np.random.default_rng(2)
    a, b = box_scene(rng, 24, 3.0), box_scene(rng, 12, 2.0, light=False)
    world = ob.OracleWorld([ob.OracleScene.from_scene(a), ob.OracleScene.from_scene(b)])
    inst = [(0, affine(np.eye(3), [0, 0, 0])), (1, affine(np.eye(3), [5.0, 0.5, -2.0])),
            (0, affine(np.eye(3), [-6.0, 1.0, 3.0])), (1, affine(np.eye(3), [0.0, -4.5, 0.0]))]
    world.set_instances(inst)
    baked, inst_of, prim_of = bake_instances([a, b], inst)
    flat = ob.OracleScene.from_scene(baked)
    rays = random_rays(rng, 20000, -8.0, 8.0)
    rays[:, 0:3] = np.round(rays[:, 0:3] * 16.0) / 16.0
    p0, t0, b0 = flat.trace(rays)
    p1, i1, t1, b1 = world.trace_instanced(rays)
    hit = p0 >= 0
    assert np.array_equal(hit, p1 >= 0)
    assert hit.mean() > 0.1
    # baked primitives are ordered by instance, then primitive: the same tie order
    assert np.array_equal(inst_of[p0[hit]], i1[hit])
    assert np.array_equal(prim_of[p0[hit]], p1[hit])
    assert np.array_equal(t0.view(np.uint32), t1.view(np.uint32))
    assert np.array_equal(b0.view(np.uint32), b1.view(np.uint32))


def test_rotated_instances_match_the_baked_scene():
    rng = np.random.default_rng(3)
    a, b = box_scene(rng, 24, 3.0), box_scene(rng, 12, 2.0, light=False)
    world = ob.OracleWorld([ob.OracleScene.from_scene(a), ob.OracleScene.from_scene(b)])
    inst = [(k % 2, m) for k, m in enumerate(_mats())]
    world.set_instances(inst)
    baked, inst_of, prim_of = bake_instances([a, b], inst)
    flat = ob.OracleScene.from_scene(baked)
    rays = random_rays(rng, 20000, -8.0, 8.0)
    p0, t0, _ = flat.trace(rays)
    p1, i1, t1, _ = world.trace_instanced(rays)
    hit = (p0 >= 0) & (p1 >= 0)
    assert hit.mean() > 0.1
    same = hit & (inst_of[np.maximum(p0, 0)] == i1) & (prim_of[np.maximum(p0, 0)] == p1)
    assert same.sum() >= 0.995 * hit.sum()   # a few rays graze edges the rounding of baking moved
    assert np.allclose(t0[same], t1[same], rtol=1e-4, atol=1e-5)
    assert np.mean((p0 >= 0) != (p1 >= 0)) < 0.005


def test_world_vertex_update_retraces():
    rng = np.random.default_rng(4)
    a = box_scene(rng, 16, 3.0)
    world = ob.OracleWorld([ob.OracleScene.from_scene(a)])
    world.set_instances([(0, affine(rotation([0, 0, 1], 20), [1.0, 0, 0]))])
    v = a.vertices.copy()
    v[:, 1] += 0.25 * np.sin(v[:, 0])
    world.update_vertices(0, v)
    moved = xr.Scene(v, a.indices, a.materials, a.ranges, a.camera)
    w2 = ob.OracleWorld([ob.OracleScene.from_scene(moved)])
    w2.set_instances([(0, affine(rotation([0, 0, 1], 20), [1.0, 0, 0]))])
    rays = random_rays(rng, 5000, -6.0, 6.0)
    r1, r2 = world.trace_instanced(rays), w2.trace_instanced(rays)
    for x, y in zip(r1, r2):
        assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))


def test_world_without_instances_traces_the_concatenated_scenes():
    """Scenes concatenated as xr_upload_scenes does (indices and material indices
    relocated) and traced as one scene when no instances are set."""
    rng = np.random.default_rng(6)
    a, b = box_scene(rng, 10, 2.0), box_scene(rng, 6, 1.5, light=False)
    world = ob.OracleWorld([ob.OracleScene.from_scene(a), ob.OracleScene.from_scene(b)])
    flat, inst_of, prim_of = bake_instances([a, b], [(0, affine(np.eye(3), [0, 0, 0])),
                                                     (1, affine(np.eye(3), [0, 0, 0]))])
    rays = random_rays(rng, 10000, -4.0, 4.0)
    p0, t0, b0 = ob.OracleScene.from_scene(flat).trace(rays)
    p1, t1, b1 = world.trace(rays)
    assert (p0 >= 0).mean() > 0.05
    assert np.array_equal(p0, p1)   # identity bakes keep the concatenation's primitive order
    assert np.array_equal(t0.view(np.uint32), t1.view(np.uint32))
    assert np.array_equal(b0.view(np.uint32), b1.view(np.uint32))
