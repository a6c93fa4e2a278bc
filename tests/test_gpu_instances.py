"""Instances, the top-level BVH and refit on the GPU against the oracle: hits of
the two-level traversal bit-exact (primitive, instance, t, barycentrics), frames
of instanced worlds bit-exact (moving instances included), identity instances
rendering exactly like the scene itself, and refitted BVHs tracing exactly like
the oracle on the moved vertices."""
import numpy as np
import pytest

import xvk_ray_gb300 as xr
from oracle import binding as ob
from tests.helpers import affine, box_scene, camera_sequence, random_rays, rotation
from tests.test_gpu_frames import _compare_frame

pytestmark = pytest.mark.gpu

XR = xr._lib


def _instances(t=0.0):
    return [(0, affine(np.eye(3), [0, 0, 0])),
            (1, affine(rotation([0, 1, 0], 30 + 40 * t) * 1.5, [2.0, -1.0 + t, 0.5])),
            (0, affine(rotation([1, 1, 0], -75) @ np.diag([0.5, 2.0, 1.0]), [-3.0, 0.25, 4.0 - 2 * t])),
            (1, affine(rotation([0, 0, 1], 10), [0.0, 3.0, -5.0]))]


def _scenes(seed=7):
    rng = np.random.default_rng(seed)
    return box_scene(rng, 24, 3.0), box_scene(rng, 12, 2.0, light=False)


def _world(scenes, inst):
    w = ob.OracleWorld([ob.OracleScene.from_scene(s) for s in scenes])
    w.set_instances(inst)
    return w


def test_instanced_trace_matches_oracle():
    scenes = _scenes()
    inst = _instances()
    world = _world(scenes, inst)
    rays = random_rays(np.random.default_rng(1), 50000, -8.0, 8.0)
    with xr.Renderer(64, 64) as r:
        r.upload_scenes(list(scenes))
        r.set_instances(inst)
        assert np.array_equal(r.instance_transforms(len(inst)).view(np.uint32), world.transforms().view(np.uint32))
        st = r.stats()
        assert st.instances == len(inst) and st.tlas_nodes >= 1
        g = r.trace_instanced(rays)
        c = world.trace_instanced(rays)
        assert (c[0] >= 0).mean() > 0.1
        for name, x, y in zip(("prim", "instance", "t", "bary"), g, c):
            assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32)), name
        ga = r.trace_instanced(rays, any_hit=True)
        ca = world.trace_instanced(rays, any_hit=True)
        assert np.array_equal(ga[0] >= 0, ca[0] >= 0)
        # the plain query reports the same primitives
        p, t, _ = r.trace(rays)
        assert np.array_equal(p, g[0])


def test_identity_instance_renders_like_the_scene():
    scene = xr.Scene.procedural(seed=3, n_objects=200, n_lights=6, extent=8.0)
    W, H = 96, 64
    ubos = camera_sequence(scene, W, H, 4, 4)
    out = []
    for use_inst in (False, True):
        with xr.Renderer(W, H) as r:
            r.set_params(xr.params_default(W, H, write_hdr=1))
            r.upload_scene(scene)
            r.build_bvh()
            if use_inst:
                r.set_instances([(0, affine(np.eye(3), [0, 0, 0]))])
            for u in ubos:
                r.render(u)
            out.append(r.read_output(XR.XR_OUT_HDR).copy())
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


@pytest.mark.parametrize("moving", [False, True])
def test_instanced_frames_match_oracle(moving):
    scenes = _scenes(11)
    W, H = 96, 72
    cam = xr._lib.XrCamera()
    cam.position[:] = [0.0, 1.0, 12.0]
    cam.yaw_deg, cam.pitch_deg, cam.fov_deg = 0.0, -5.0, 60.0
    view = xr.Scene(scenes[0].vertices, scenes[0].indices, scenes[0].materials, scenes[0].ranges, cam)
    ubos = camera_sequence(view, W, H, 5, 4)
    p = xr.params_default(W, H, write_hdr=1, write_pt=1)
    world = _world(scenes, _instances(0.0))
    o = ob.OracleRenderer(world, p)
    with xr.Renderer(W, H) as r:
        r.set_params(p)
        r.upload_scenes(list(scenes))
        for f, u in enumerate(ubos):
            inst = _instances(0.1 * f if moving else 0.0)
            if moving or f == 0:
                r.set_instances(inst)
                world.set_instances(inst)
            r.render(u)
            o.render(u)
            _compare_frame(r, o, False, f"frame {f}")


def test_bounded_camera_rays_in_an_instanced_world():
    """Camera rays are first bounded just past their pixel's previous visible point in
    instanced worlds too; a ray with nothing inside the bound is traced again from the
    top-level root.  Moving instances and a camera that steps back and turns send many
    rays through that second trace; the frames stay bit-identical to the oracle."""
    rng = np.random.default_rng(41)
    scenes = (box_scene(rng, 300, 4.0), box_scene(rng, 12, 2.0, light=False))
    W, H = 96, 72
    cam = xr._lib.XrCamera()
    cam.position[:] = [0.0, 1.0, 12.0]
    cam.yaw_deg, cam.pitch_deg, cam.fov_deg = 0.0, -5.0, 60.0
    view = xr.Scene(scenes[0].vertices, scenes[0].indices, scenes[0].materials, scenes[0].ranges, cam)

    def move(f, c):
        if f == 2:
            c.position[2] += 3.0
        elif f == 3:
            c.yaw_deg += 60.0

    ubos = camera_sequence(view, W, H, 5, 4, move=move)
    p = xr.params_default(W, H, write_hdr=1, write_pt=1)
    world = _world(scenes, _instances(0.0))
    o = ob.OracleRenderer(world, p)
    with xr.Renderer(W, H) as r:
        r.set_params(p)
        r.upload_scenes(list(scenes))
        assert r.stats().bvh_nodes >= 256   # large enough for the bounded camera-ray kernel
        for f, u in enumerate(ubos):
            inst = _instances(0.1 * f)
            r.set_instances(inst)
            world.set_instances(inst)
            r.render(u)
            o.render(u)
            _compare_frame(r, o, False, f"frame {f}")


def test_refit_traces_like_the_moved_scene():
    scene = xr.Scene.procedural(seed=9, n_objects=300, n_lights=4, extent=8.0)
    rng = np.random.default_rng(5)
    rays = random_rays(rng, 50000, -8.0, 8.0)
    v = scene.vertices.copy()
    v[:, 1] += 0.3 * np.sin(0.7 * v[:, 0]) * np.cos(0.5 * v[:, 2])
    moved = xr.Scene(v, scene.indices, scene.materials, scene.ranges, scene.camera)
    oracle = ob.OracleScene.from_scene(moved)
    with xr.Renderer(64, 64) as r:
        r.upload_scene(scene)
        r.build_bvh()
        r.update_vertices(0, v)
        assert r.stats().ms_refit > 0.0
        g = r.trace(rays)
        c = oracle.trace(rays)
        assert (c[0] >= 0).mean() > 0.2
        for name, x, y in zip(("prim", "t", "bary"), g, c):
            assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32)), name
        # and under an instance
        inst = [(0, affine(rotation([0, 1, 0], 25), [0.5, 0.0, -1.0]))]
        r.set_instances(inst)
        world = ob.OracleWorld([oracle])
        world.set_instances(inst)
        g = r.trace_instanced(rays)
        c = world.trace_instanced(rays)
        for name, x, y in zip(("prim", "instance", "t", "bary"), g, c):
            assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32)), name


def test_instance_errors():
    scenes = _scenes()
    with xr.Renderer(32, 32) as r:
        r.upload_scenes(list(scenes))
        with pytest.raises(xr.XrError):
            r.set_instances([(2, affine(np.eye(3), [0, 0, 0]))])
        with pytest.raises(xr.XrError):
            r.set_instances([(0, affine(np.diag([1.0, 0.0, 1.0]), [0, 0, 0]))])
        r.set_instances([(0, affine(np.eye(3), [0, 0, 0]))])
        r.set_instances([])
        assert r.stats().instances == 0
        p, inst, t, _ = r.trace_instanced(random_rays(np.random.default_rng(0), 100, -3, 3))
        assert np.all(inst == -1)


def test_instanced_views_match_single_views():
    """With instances set every view renders the instanced world; each view of a
    two-view frame is bit-identical to rendering it alone."""
    scenes = _scenes(13)
    inst = _instances(0.0)
    cam = xr._lib.XrCamera()
    cam.position[:] = [0.0, 1.0, 12.0]
    cam.yaw_deg, cam.pitch_deg, cam.fov_deg = 0.0, -5.0, 60.0
    base = xr.Scene(scenes[0].vertices, scenes[0].indices, scenes[0].materials, scenes[0].ranges, cam)
    views = [(0, 64, 48), (1, 40, 56)]

    def mover(dyaw):
        def f(frame, c):
            c.yaw_deg += dyaw
        return f

    seqs = [camera_sequence(base, w, h, 3, 4, move=mover(0.3 * (k + 1))) for k, (_, w, h) in enumerate(views)]
    alone = []
    for k, (_, w, h) in enumerate(views):
        with xr.Renderer(w, h) as r:
            r.set_params(xr.params_default(w, h, write_hdr=1))
            r.upload_scenes(list(scenes))
            r.set_instances(inst)
            for u in seqs[k]:
                r.render(u)
            alone.append(r.read_output(XR.XR_OUT_HDR).copy())
    r = xr.Renderer(8, 8)
    r.upload_scenes(list(scenes))
    r.set_views(views, xr.params_default(8, 8, write_hdr=1))
    r.set_instances(inst)
    for f in range(3):
        r.render_views([seqs[v][f] for v in range(len(views))])
    for k in range(len(views)):
        got = r.read_view_output(k, XR.XR_OUT_HDR)
        assert np.array_equal(got.view(np.uint32), alone[k].view(np.uint32)), f"view {k}"
    r.close()


def test_frames_across_a_refit_match_oracle():
    """Frames before and after new vertex positions (the temporal pass reprojecting
    across the change) against the oracle rebuilt on the moved geometry."""
    rng = np.random.default_rng(21)
    scene = box_scene(rng, 24, 3.0)
    W, H = 80, 60
    cam = xr._lib.XrCamera()
    cam.position[:] = [0.0, 0.5, 10.0]
    cam.yaw_deg, cam.pitch_deg, cam.fov_deg = 0.0, -3.0, 60.0
    view = xr.Scene(scene.vertices, scene.indices, scene.materials, scene.ranges, cam)
    ubos = camera_sequence(view, W, H, 5, 4)
    p = xr.params_default(W, H, write_hdr=1, write_pt=1)
    world = ob.OracleWorld([ob.OracleScene.from_scene(scene)])   # no instances: traced as one scene
    o = ob.OracleRenderer(world, p)
    moved = scene.vertices.copy()
    moved[:, 1] += 0.2 * np.sin(0.9 * moved[:, 0])
    with xr.Renderer(W, H) as r:
        r.set_params(p)
        r.upload_scene(scene)
        r.build_bvh()
        for f, u in enumerate(ubos):
            if f == 2:
                r.update_vertices(0, moved)
                world.update_vertices(0, moved)
            r.render(u)
            o.render(u)
            _compare_frame(r, o, False, f"frame {f}")


def test_instances_of_empty_and_one_triangle_scenes():
    rng = np.random.default_rng(17)
    boxes = box_scene(rng, 8, 2.0)
    tri = xr.Scene(np.array([[-1, -1, 0, 0, 0, 1, 0, 0, 0], [1, -1, 0, 0, 0, 1, 0, 0, 0],
                             [0, 1, 0, 0, 0, 1, 0, 0, 0]], np.float32),
                   np.array([0, 1, 2], np.uint32), boxes.materials[:1].copy(), np.zeros((1, 2), np.uint32),
                   boxes.camera)
    empty = xr.Scene(np.zeros((0, 9), np.float32), np.zeros(0, np.uint32), boxes.materials[:1].copy(),
                     np.zeros((1, 2), np.uint32), boxes.camera)
    scenes = [boxes, tri, empty]
    inst = [(0, affine(np.eye(3), [0, 0, 0])), (1, affine(rotation([0, 1, 0], 40) * 2.0, [3.0, 0.0, 1.0])),
            (2, affine(np.eye(3), [0.0, 5.0, 0.0])), (1, affine(np.eye(3), [-3.0, 1.0, -1.0]))]
    world = _world(scenes, inst)
    rays = random_rays(np.random.default_rng(3), 20000, -6.0, 6.0)
    with xr.Renderer(32, 32) as r:
        r.upload_scenes(scenes)
        r.set_instances(inst)
        g = r.trace_instanced(rays)
        c = world.trace_instanced(rays)
        assert np.any(c[1] == 1) and np.any(c[1] == 3)   # the one-triangle instances are hit
        for name, x, y in zip(("prim", "instance", "t", "bary"), g, c):
            assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32)), name


def test_many_instances_match_oracle():
    """600 instances: a top-level BVH several levels deep (the tests above fit in one
    node), rotated and scaled copies scattered over a 40-unit cube."""
    rng = np.random.default_rng(31)
    box = box_scene(rng, 1, 1.0, light=False)
    inst = []
    for k in range(600):
        R = rotation(rng.normal(size=3), float(rng.uniform(0, 360))) * float(rng.uniform(0.3, 1.5))
        inst.append((0, affine(R, rng.uniform(-20.0, 20.0, 3))))
    world = _world([box], inst)
    # rays from random origins aimed at random instances (most of them hit something)
    rr = np.random.default_rng(2)
    rays = random_rays(rr, 8000, -22.0, 22.0)
    pick = rr.integers(0, len(inst), 8000)
    vtx = box.vertices[rr.integers(0, box.vertices.shape[0], 8000), 0:3].astype(np.float64)
    mats = np.array([m for _, m in inst], np.float64)[pick]
    targets = np.einsum("nij,nj->ni", mats[:, :, :3], vtx) + mats[:, :, 3] + rr.normal(0, 0.05, (8000, 3))
    d = targets - rays[:, 0:3]
    rays[:, 4:7] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    with xr.Renderer(32, 32) as r:
        r.upload_scenes([box])
        r.set_instances(inst)
        assert r.stats().tlas_nodes > 8
        g = r.trace_instanced(rays)
        c = world.trace_instanced(rays)
        assert (c[0] >= 0).mean() > 0.3
        for name, x, y in zip(("prim", "instance", "t", "bary"), g, c):
            assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32)), name
        ga = r.trace_instanced(rays, any_hit=True)
        ca = world.trace_instanced(rays, any_hit=True)
        assert np.array_equal(ga[0] >= 0, ca[0] >= 0)


def test_vertex_update_errors():
    scene = xr.Scene.cornell()
    with xr.Renderer(32, 32) as r:
        r.upload_scene(scene)
        r.build_bvh()
        with pytest.raises(xr.XrError):
            r.update_vertices(0, scene.vertices[:-1])          # the count must stay
        with pytest.raises(xr.XrError):
            r.update_vertices(1, scene.vertices)               # no such scene
        bad = scene.vertices.copy()
        bad[0, 0] = np.nan
        with pytest.raises(xr.XrError):
            r.update_vertices(0, bad)
        r.update_vertices(0, scene.vertices)                   # unchanged geometry refits fine


def test_deferred_top_level_and_reused_arrays_match_oracle():
    """Vertex updates of an instanced scene rebuild the top level once, at the next
    trace or frame; instance lists that shrink and grow reuse or replace the
    instance arrays. Every step traced and rendered bit-exact against the oracle."""
    scenes = _scenes(13)
    W, H = 64, 48
    cam = xr._lib.XrCamera()
    cam.position[:] = [0.0, 1.0, 12.0]
    cam.yaw_deg, cam.pitch_deg, cam.fov_deg = 0.0, -5.0, 60.0
    view = xr.Scene(scenes[0].vertices, scenes[0].indices, scenes[0].materials, scenes[0].ranges, cam)
    ubos = camera_sequence(view, W, H, 6, 4)
    p = xr.params_default(W, H, write_hdr=1, write_pt=1)
    inst = _instances(0.0)
    world = _world(scenes, inst)
    o = ob.OracleRenderer(world, p)
    rays = random_rays(np.random.default_rng(4), 20000, -8.0, 8.0)

    def moved(f):
        v = scenes[1].vertices.copy()
        v[:, 1] += 0.15 * np.sin(1.3 * v[:, 0] + f)
        return v

    extra = [(1, affine(rotation([1, 0, 0], 20), [4.0, 0.5, 2.0])), (0, affine(np.eye(3) * 0.5, [-4.0, 2.0, 1.0]))]
    steps = ["update", "update twice", "shrink", "grow", "update"]
    with xr.Renderer(W, H) as r:
        r.set_params(p)
        r.upload_scenes(list(scenes))
        r.set_instances(inst)
        r.render(ubos[0])
        o.render(ubos[0])
        _compare_frame(r, o, False, "frame 0")
        for f, step in enumerate(steps, start=1):
            if step.startswith("update"):
                if step == "update twice":
                    r.update_vertices(1, moved(f + 0.5))
                r.update_vertices(1, moved(f))
                world.update_vertices(1, moved(f))
            else:
                inst = inst[:2] if step == "shrink" else inst + extra
                r.set_instances(inst)
                world.set_instances(inst)
                assert r.stats().instances == len(inst)
            # the stale top level is rebuilt by whichever comes first: the trace, or (last step) the frame
            if f == len(steps):
                r.render(ubos[f])
                o.render(ubos[f])
                _compare_frame(r, o, False, f"frame {f} ({step})")
            g = r.trace_instanced(rays)
            c = world.trace_instanced(rays)
            for name, x, y in zip(("prim", "instance", "t", "bary"), g, c):
                assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32)), f"{step}: {name}"
            if f < len(steps):
                r.render(ubos[f])
                o.render(ubos[f])
                _compare_frame(r, o, False, f"frame {f} ({step})")
