"""xr_trace_rays_noalloc: ray queries for callers that cannot allocate device memory.

An engine that owns every byte of device memory through its own allocator, or a
real-time loop that must not pay for an allocation's implicit synchronisation,
cannot let the library cudaMalloc per query the way xr_trace_rays stages its
rays.  The no-alloc entry point stages through a fixed device array of the
library instead.  This file runs last (pytest collects files by name) and
checks, through the C ABI:

* two calls in a row return what the oracle's traversal returns (and what
  xr_trace_rays returns), closest-hit and any-hit;
* the device's free memory is the same before and after calls (nothing is
  allocated, once the library's module is loaded);
* oversize batches are refused before anything is written;
* an instanced world traces through the two-level BVH, and a world whose top
  level went stale after xr_update_vertices is refused (its rebuild would
  allocate) until a frame or an allocating query rebuilds it.
"""
import numpy as np
import pytest

import xvk_ray_gb300 as xr
from oracle import binding as ob
from tests.helpers import affine, random_rays, rotation

pytestmark = pytest.mark.gpu

L = xr._lib
MAX_RAYS = 65536


def _noalloc(r, rays, any_hit):
    lib = L.load()
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    prim = np.full(n, -7, np.int32)
    t = np.full(n, np.nan, np.float32)
    bary = np.full((n, 2), np.nan, np.float32)
    st = lib.xr_trace_rays_noalloc(r.ctx, rays.ctypes.data, n, 1 if any_hit else 0, prim.ctypes.data,
                                   t.ctypes.data, bary.ctypes.data)
    return st, prim, t, bary


def _same(got, expect):
    gp, gt, gb = got
    ep, et, eb = expect[0], expect[1], expect[2]
    assert np.array_equal(gp, ep)
    hit = gp >= 0
    assert np.array_equal(gt[hit].view(np.uint32), np.asarray(et)[hit].view(np.uint32))
    assert np.array_equal(gb[hit].view(np.uint32), np.asarray(eb)[hit].view(np.uint32))


def _free_bytes() -> int:
    import torch
    return int(torch.cuda.mem_get_info(0)[0])


def test_noalloc_matches_oracle_two_calls():
    scene = xr.Scene.procedural(seed=9, n_objects=512, extent=10.0)
    oracle = ob.OracleScene.from_scene(scene)
    rng = np.random.default_rng(21)
    batches = [random_rays(rng, MAX_RAYS, [-12, 0.0, -12], [12, 4.0, 12]),
               random_rays(rng, 40000, [-12, 0.0, -12], [12, 4.0, 12])]
    with xr.Renderer(8, 8) as r:
        r.set_params(xr.params_default(8, 8))
        r.upload_scene(scene)
        r.build_bvh()
        for any_hit in (False, True):
            for rays in batches:
                expect = oracle.trace(rays, any_hit)
                assert (expect[0] >= 0).mean() > 0.2
                for _ in range(2):                        # two calls in a row share the array
                    st, *got = _noalloc(r, rays, any_hit)
                    assert st == L.XR_OK, L.load().xr_last_error(r.ctx)
                    if any_hit:
                        assert np.array_equal(got[0] >= 0, expect[0] >= 0)
                    else:
                        _same(tuple(got), expect)
                if not any_hit:
                    _same(tuple(r.trace(rays, False)), expect)   # the allocating entry point agrees


def test_noalloc_allocates_nothing():
    scene = xr.Scene.procedural(seed=3, n_objects=256, extent=8.0)
    rays = random_rays(np.random.default_rng(4), MAX_RAYS, [-10, 0.0, -10], [10, 4.0, 10])
    with xr.Renderer(8, 8) as r:
        r.set_params(xr.params_default(8, 8))
        r.upload_scene(scene)
        r.build_bvh()
        st, *_ = _noalloc(r, rays, False)                 # loads the module holding the fixed array
        assert st == L.XR_OK
        before = _free_bytes()
        for any_hit in (False, True, False):
            st, *_ = _noalloc(r, rays, any_hit)
            assert st == L.XR_OK, L.load().xr_last_error(r.ctx)
        assert _free_bytes() == before


def test_noalloc_refuses_oversize_batch():
    scene = xr.Scene.cornell()
    with xr.Renderer(8, 8) as r:
        r.set_params(xr.params_default(8, 8))
        r.upload_scene(scene)
        r.build_bvh()
        rays = random_rays(np.random.default_rng(2), MAX_RAYS + 1, [-1, 0, -1], [1, 2, 1])
        st, prim, _, _ = _noalloc(r, rays, False)
        assert st == L.XR_ERR_INVALID_ARGUMENT
        assert b"65536" in L.load().xr_last_error(r.ctx)
        assert np.all(prim == -7)                         # nothing was written


def test_noalloc_instanced_world_and_stale_top_level():
    scene = xr.Scene.procedural(seed=5, n_objects=120, n_lights=2, extent=4.0)
    inst = [(0, affine(np.eye(3), [0.0, 0.0, 0.0])),
            (0, affine(rotation([0, 1, 0], 35.0) * 0.75, [6.0, 0.5, -2.0]))]
    rays = random_rays(np.random.default_rng(8), 30000, [-6, 0.0, -6], [10, 3.0, 6])
    with xr.Renderer(8, 8) as r:
        r.upload_scenes([scene])
        r.set_instances(inst)
        world = ob.OracleWorld([ob.OracleScene.from_scene(scene)])
        world.set_instances(inst)
        expect = world.trace_instanced(rays)
        assert (expect[0] >= 0).mean() > 0.1
        st, *got = _noalloc(r, rays, False)
        assert st == L.XR_OK, L.load().xr_last_error(r.ctx)
        _same(tuple(got), (expect[0], expect[2], expect[3]))
        # move the scene's vertices: the top level goes stale and would need a rebuild
        v = scene.vertices.copy()
        v[:, 1] += 0.25
        r.update_vertices(0, v)
        st, prim, _, _ = _noalloc(r, rays, False)
        assert st == L.XR_ERR_STATE
        assert b"stale" in L.load().xr_last_error(r.ctx)
        assert np.all(prim == -7)
        r.trace_instanced(rays[:16])                      # an allocating query rebuilds the top level
        moved = xr.Scene(v, scene.indices, scene.materials, scene.ranges, scene.camera)
        world = ob.OracleWorld([ob.OracleScene.from_scene(moved)])
        world.set_instances(inst)
        expect = world.trace_instanced(rays)
        for _ in range(2):
            st, *got = _noalloc(r, rays, False)
            assert st == L.XR_OK, L.load().xr_last_error(r.ctx)
            _same(tuple(got), (expect[0], expect[2], expect[3]))
