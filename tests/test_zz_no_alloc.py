"""xr_trace_rays_noalloc: ray queries for callers that cannot allocate device memory.

An engine that owns every byte of device memory through its own allocator, or a
real-time loop that must not pay for an allocation's implicit synchronisation,
cannot let the library cudaMalloc per query the way xr_trace_rays stages its
rays.  The no-alloc entry point stages through a fixed device array of the
library instead.  This file runs last (pytest collects files by name) and
checks, through the C ABI, that two calls in a row return exactly what
xr_trace_rays returns, and that oversize batches are refused.
"""
import ctypes as C

import numpy as np
import pytest

import xvk_ray_gb300 as xr
from tests.helpers import random_rays

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


def _same(a, b):
    ap, at, ab = a
    bp, bt, bb = b
    assert np.array_equal(ap, bp)
    hit = ap >= 0
    assert np.array_equal(at[hit].view(np.uint32), bt[hit].view(np.uint32))
    assert np.array_equal(ab[hit].view(np.uint32), bb[hit].view(np.uint32))


def test_noalloc_matches_trace_rays_two_calls():
    scene = xr.Scene.procedural(seed=9, n_objects=512, extent=10.0)
    rng = np.random.default_rng(21)
    batches = [random_rays(rng, MAX_RAYS, [-12, 0.0, -12], [12, 4.0, 12]),
               random_rays(rng, 40000, [-12, 0.0, -12], [12, 4.0, 12])]
    with xr.Renderer(8, 8) as r:
        r.set_params(xr.params_default(8, 8))
        r.upload_scene(scene)
        r.build_bvh()
        for any_hit in (False, True):
            for rays in batches:
                expect = r.trace(rays, any_hit)          # xr_trace_rays (allocates its staging)
                for _ in range(2):                        # two calls in a row share the array
                    st, *got = _noalloc(r, rays, any_hit)
                    assert st == L.XR_OK, L.load().xr_last_error(r.ctx)
                    if any_hit:
                        assert np.array_equal(got[0] >= 0, expect[0] >= 0)
                    else:
                        _same(tuple(got), expect)


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
