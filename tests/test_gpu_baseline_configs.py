"""Parity at the benchmark's own configurations, against the oracle.

* Configuration 0 as stated: the procedural Cornell box (5 wall quads and two
  boxes rotated 15 / -18 degrees: 34 triangles, plus the two triangles of the
  0.25-unit^2 area light), 256 x 256, 8 frames of a static camera, 1 spp, depth
  4, the benchmark settings (temporal M cap 20, 5 neighbours in 30 px, spatial
  shadow rays, seed 1): every sample and reservoir field and the linear image
  bit-identical, every frame.
* The 1080p benchmark scene (seed 1, 4096 objects, 16 lights: 998,442 triangles
  in a 163,048-node 8-wide BVH): primitive, t and barycentrics of one camera ray
  per pixel at 1920 x 1080 and of 1M random rays, bit-identical to the oracle's
  traversal; any-hit queries agree on hit or miss.
* That scene's frames along the benchmark's camera path (0.01 units and 0.2
  degrees per frame) at 240 x 135 -- the benchmark's scene, camera and settings
  at 1/64 of the pixels -- 4 frames, field by field.
"""
import numpy as np
import pytest

import xvk_ray_gb300 as xr
from oracle import binding as ob
from tests.helpers import camera_sequence
from tests.test_gpu_frames import _compare_frame, _setup

pytestmark = pytest.mark.gpu
XR = xr._lib

BENCH_SCENE = dict(seed=1, n_objects=4096, n_lights=16, extent=40.0, sphere_subdiv=2)


def _bench_path(f, cam):
    cam.position[2] -= 0.01
    cam.yaw_deg += 0.2


def test_config0_cornell_256_eight_static_frames():
    scene = xr.Scene.cornell()
    assert scene.n_triangles == 34 + 2       # walls and boxes, then the light quad
    W = H = 256
    p = xr.params_default(W, H, write_hdr=1, write_pt=1)
    assert (p.m_cap_temporal, p.n_neighbours, p.radius_px, p.visibility, p.seed) == (20, 5, 30.0, 1, 1)
    r, o = _setup(scene, p)
    with r:
        for f, u in enumerate(camera_sequence(scene, W, H, 8, 4)):
            r.render(u)
            o.render(u)
            _compare_frame(r, o, False, f"frame {f}")
        assert r.stats().shadow_rays > 0
        assert np.array_equal(r.read_output(XR.XR_OUT_PT).view(np.uint32), o.read(ob.BUF_PT).view(np.uint32))


def _camera_rays(ubo, W, H) -> np.ndarray:
    """One ray through each pixel centre (o, tmin 1e-4, d, tmax 1e4)."""
    vi = np.array(ubo.view_inverse, np.float64).reshape(4, 4).T      # glm column-major
    pi = np.array(ubo.projection_inverse, np.float64).reshape(4, 4).T
    ys, xs = np.mgrid[0:H, 0:W]
    uv = np.stack([(xs.reshape(-1) + 0.5) / W * 2 - 1, (ys.reshape(-1) + 0.5) / H * 2 - 1], 1)
    tgt = np.concatenate([uv, np.ones((uv.shape[0], 2))], 1) @ pi.T
    t3 = tgt[:, :3] / np.linalg.norm(tgt[:, :3], axis=1, keepdims=True)
    d = np.concatenate([t3, np.zeros((t3.shape[0], 1))], 1) @ vi.T
    d = d[:, :3] / np.linalg.norm(d[:, :3], axis=1, keepdims=True)
    o = vi[:3, 3]
    rays = np.zeros((d.shape[0], 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = 1e-4
    rays[:, 4:7] = d
    rays[:, 7] = 1e4
    return rays


def _random_rays(rng, n) -> np.ndarray:
    o = rng.uniform([-42.0, 0.02, -42.0], [42.0, 6.0, 42.0], (n, 3))
    d = rng.normal(size=(n, 3))
    d[:, 1] -= 0.3                                   # more rays toward the ground and the objects
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = 1e-4
    rays[:, 4:7] = d
    rays[:, 7] = 1e4
    return rays


def test_benchmark_scene_hits_bit_exact():
    scene = xr.Scene.procedural(**BENCH_SCENE)
    assert scene.n_triangles == 998442
    ubo = camera_sequence(scene, 1920, 1080, 1, 4, move=_bench_path)[0]
    batches = {"camera rays 1920x1080": _camera_rays(ubo, 1920, 1080),
               "1M random rays": _random_rays(np.random.default_rng(17), 1 << 20)}
    oracle = ob.OracleScene.from_scene(scene)
    with xr.Renderer(8, 8) as r:
        r.upload_scene(scene)
        r.build_bvh()
        st = r.stats()
        assert (st.bvh_nodes, st.bvh_depth) == (163048, 12)
        for name, rays in batches.items():
            g = r.trace(rays)
            c = oracle.trace(rays)
            assert (c[0] >= 0).mean() > 0.5, name
            assert np.array_equal(g[0], c[0]), f"{name}: primitive"
            hit = c[0] >= 0
            assert np.array_equal(np.asarray(g[1])[hit].view(np.uint32), np.asarray(c[1])[hit].view(np.uint32)), \
                f"{name}: t"
            assert np.array_equal(np.asarray(g[2])[hit].view(np.uint32), np.asarray(c[2])[hit].view(np.uint32)), \
                f"{name}: barycentrics"
            ga = r.trace(rays, any_hit=True)
            ca = oracle.trace(rays, any_hit=True)
            assert np.array_equal(ga[0] >= 0, ca[0] >= 0), f"{name}: any hit"


def test_benchmark_scene_frames_240x135():
    scene = xr.Scene.procedural(**BENCH_SCENE)
    W, H = 240, 135
    p = xr.params_default(W, H, write_hdr=1)
    r, o = _setup(scene, p)
    with r:
        for f, u in enumerate(camera_sequence(scene, W, H, 4, 4, move=_bench_path)):
            r.render(u)
            o.render(u)
            _compare_frame(r, o, False, f"frame {f}")
        assert r.stats().shadow_rays > 0
