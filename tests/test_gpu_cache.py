"""Learned radiance cache kernels (tcgen05 BF16 MMAs, FP32 accumulation) against the oracle.

Inputs to the network are bit-identical on both sides (same encoding arithmetic);
the oracle accumulates dot products in double and rounds where the kernels round,
so what differs is the FP32 accumulation order inside the tensor-core MMAs and of
the atomic gradient sums: outputs and gradients are compared by relative norm
error (tolerances below), Adam and initialisation bit-exactly.
"""
import numpy as np
import pytest

import xvk_ray_gb300 as xr
from xvk_ray_gb300 import _lib as L
from oracle import binding as ob
from tests.test_oracle_cache import _samples

pytestmark = pytest.mark.gpu

LO, INV = [-1.0, -1.0, -1.0], 0.5
OUT_TOL = 5e-3      # relative norm error of predictions (bf16 activations, FP32 MMA accumulation)
GRAD_TOL = 2e-2     # relative norm error of gradients (additionally, FP32 atomics order)


def _pair(seed=3):
    r = xr.Renderer(8, 8)
    r.set_params(xr.params_default(8, 8))
    r.cache.reset(seed)
    r.cache.set_bounds(LO, INV)
    oc = ob.OracleCache(seed)
    oc.set_bounds(LO, INV)
    return r, oc


def _shared_state(r, oc, seed=0):
    """Table values of a trained cache's magnitude, identical on both sides."""
    rng = np.random.default_rng(seed)
    g = oc.param(ob.NRC_GRID)
    g[:] = (rng.standard_normal(g.size) * 0.3).astype(np.float32)
    r.cache.write(L.XR_CACHE_GRID, g)
    r.cache.write(L.XR_CACHE_MLP, oc.param(ob.NRC_MLP))


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(np.asarray(b, np.float64)), 1e-30))


def test_init_matches_oracle():
    r, oc = _pair(3)
    with r:
        assert np.array_equal(r.cache.read(L.XR_CACHE_MLP), oc.param(ob.NRC_MLP))
        assert np.array_equal(r.cache.read(L.XR_CACHE_GRID), oc.param(ob.NRC_GRID))
        assert r.cache.stats().steps == 0


@pytest.mark.parametrize("n", [1, 127, 1000, 8192])
def test_query_matches_oracle(n):
    r, oc = _pair(4)
    with r:
        _shared_state(r, oc)
        s = _samples(np.random.default_rng(n), n)
        gpu = r.cache.query(s)
    ref = oc.infer(ob.pack_cache_samples(s))
    assert np.all(np.isfinite(gpu))
    assert _rel(gpu, ref) < OUT_TOL, _rel(gpu, ref)


# 16,384 uniform samples overflow the per-chunk shared-memory sums of the finer
# aggregated levels (more distinct entries per 2,048-sample chunk than slots), so
# both the summed and the direct paths of the table gradient are covered.
@pytest.mark.parametrize("n", [1024, 16384])
def test_gradients_match_oracle(n):
    r, oc = _pair(5)
    with r:
        _shared_state(r, oc, seed=1)
        s = _samples(np.random.default_rng(7), n)
        loss = r.cache.train(s, apply=False)
        gw = r.cache.read(L.XR_CACHE_MLP_GRAD)
        gg = r.cache.read(L.XR_CACHE_GRID_GRAD)
    ref_loss = oc.backward(ob.pack_cache_samples(s), s["target"], exact=False, loss_kind=0)
    assert abs(loss - ref_loss) <= 1e-3 * abs(ref_loss)
    ow, og = oc.param(ob.NRC_MLP_GRAD), oc.param(ob.NRC_GRID_GRAD)
    for l in range(5):
        lo, hi = l * 4096, l * 4096 + (4096 if l < 4 else 1024)
        assert _rel(gw[lo:hi], ow[lo:hi]) < GRAD_TOL, (l, _rel(gw[lo:hi], ow[lo:hi]))
    touched = np.flatnonzero(og)
    assert len(touched) > 10000
    assert _rel(gg, og) < GRAD_TOL, _rel(gg, og)
    # no gradient outside the touched entries
    assert np.count_nonzero(gg[np.setdiff1d(np.arange(0, gg.size, 101), touched)]) == 0


def test_adam_step_bit_exact():
    r, oc = _pair(6)
    rng = np.random.default_rng(2)
    p1 = p2 = np.float32(1.0)
    with r:
        for step in (1, 2):
            gw = rng.standard_normal(17408).astype(np.float32)
            gg = np.zeros(16 * (1 << 19) * 2, np.float32)
            idx = rng.choice(gg.size, 20000, replace=False)
            gg[idx] = rng.standard_normal(20000).astype(np.float32)
            r.cache.write(L.XR_CACHE_MLP_GRAD, gw)
            r.cache.write(L.XR_CACHE_GRID_GRAD, gg)
            r.cache.step()
            oc.param(ob.NRC_MLP_GRAD)[:] = gw
            oc.param(ob.NRC_GRID_GRAD)[:] = gg
            p = r.cache.params()
            # bias correction as the device keeps it: FP32 running powers of beta
            p1, p2 = np.float32(p1 * np.float32(p.beta1)), np.float32(p2 * np.float32(p.beta2))
            bc1, bc2 = np.float32(np.float32(1.0) - p1), np.float32(np.float32(1.0) - p2)
            oc.adam(p.learning_rate, p.beta1, p.beta2, p.epsilon, bc1, bc2)
            for which, ow in ((L.XR_CACHE_MLP, ob.NRC_MLP), (L.XR_CACHE_MLP_M, ob.NRC_MLP_M),
                              (L.XR_CACHE_MLP_V, ob.NRC_MLP_V), (L.XR_CACHE_GRID, ob.NRC_GRID),
                              (L.XR_CACHE_GRID_M, ob.NRC_GRID_M), (L.XR_CACHE_GRID_V, ob.NRC_GRID_V)):
                assert np.array_equal(r.cache.read(which), oc.param(ow)), (step, which)
            assert np.count_nonzero(r.cache.read(L.XR_CACHE_MLP_GRAD)) == 0
            assert np.count_nonzero(r.cache.read(L.XR_CACHE_GRID_GRAD)) == 0
        assert r.cache.stats().steps == 2


def _field(s):
    """A smooth radiance field over position / normal / direction for training."""
    p, n, w = s["pos"], s["normal"], s["wo"]
    base = 0.6 + 0.4 * np.sin(3.0 * p[:, 0]) * np.cos(2.0 * p[:, 2]) + 0.2 * p[:, 1:2].repeat(1, 1)[:, 0]
    rgb = np.stack([base * (0.7 + 0.3 * n[:, 1]), base * s["albedo"][:, 1], 0.5 * base * (1.0 + w[:, 2] * 0.3)], 1)
    return np.clip(rgb, 0.0, None).astype(np.float32)


def _rel_l2(y, t):
    return float(np.mean((y - t) ** 2 / (t ** 2 + 0.01)))


def test_training_converges():
    rng = np.random.default_rng(11)
    held = _samples(rng, 4096)
    held["target"] = _field(held)
    with xr.Renderer(8, 8) as r:
        r.set_params(xr.params_default(8, 8))
        r.cache.reset(9)
        r.cache.set_bounds(LO, INV)
        before = _rel_l2(r.cache.query(held), held["target"])
        losses = []
        for _ in range(300):
            s = _samples(rng, 4096)
            s["target"] = _field(s)
            losses.append(r.cache.train(s, apply=True))
        after = _rel_l2(r.cache.query(held), held["target"])
        st = r.cache.stats()
    assert st.steps == 300
    assert np.all(np.isfinite(losses))
    assert np.mean(losses[-20:]) < 0.1 * np.mean(losses[:5])
    assert after < 0.1 * before, (before, after)


def test_checkpoint_resume_is_exact():
    """A trained cache saved with checkpoint() (arrays 0..7, the Adam step count and the
    encoding bounds) and restored into a fresh context predicts bit-identically, and the next Adam step
    (which reads the step count for its bias correction) gives bit-identical state."""
    r, oc = _pair(5)
    with r:
        _shared_state(r, oc)
        s = _samples(np.random.default_rng(7), 4096)
        for _ in range(3):
            r.cache.train(s)
        r.cache.train(s, apply=False)   # gradients pending, not yet applied
        state = r.cache.checkpoint()
        assert int(state[L.XR_CACHE_ADAM_STEP][0]) == 3 == r.cache.stats().steps
        q = s[:1000]
        before = r.cache.query(q)
        with xr.Renderer(8, 8) as r2:
            r2.set_params(xr.params_default(8, 8))
            r2.cache.reset(99)                 # a different initialisation, overwritten below
            r2.cache.set_bounds([0.0, 0.0, 0.0], 0.25)   # another scene cube: restore() brings LO, INV back
            r2.cache.restore(state)
            st2 = r2.cache.stats()
            assert st2.steps == 3
            assert list(st2.bounds_lo) == LO and st2.inv_extent == INV
            for w in range(8):
                assert np.array_equal(r2.cache.read(w), state[w]), w
            assert np.array_equal(r2.cache.query(q), before)
            r.cache.step()
            r2.cache.step()
            for w in (L.XR_CACHE_MLP, L.XR_CACHE_GRID, L.XR_CACHE_MLP_M, L.XR_CACHE_MLP_V, L.XR_CACHE_GRID_M,
                      L.XR_CACHE_GRID_V):
                assert np.array_equal(r2.cache.read(w), r.cache.read(w)), w
            assert np.array_equal(r2.cache.query(q), r.cache.query(q))
        with pytest.raises(xr.XrError):
            r.cache.write(L.XR_CACHE_ADAM_STEP, np.zeros(2, np.uint32))   # one uint32 only


def test_bounded_tensor_core_wait_gives_up():
    """The failure path of the cache kernels' bounded waits: a CTA holding tensor
    memory waits on an mbarrier phase that nothing completes (no MMA issued), gives
    up after 2 ms, raises XR_DEVFLAG_MMA_TIMEOUT and frees its tensor memory; the
    call reports XR_ERR_TIMEOUT and the context goes on rendering."""
    lib = L.load()
    scene = xr.Scene.cornell()
    with xr.Renderer(32, 32) as r:
        r.set_params(xr.params_default(32, 32))
        r.upload_scene(scene)
        r.build_bvh()
        assert r.stats().error_flags == 0
        st = lib.xr_cache_selftest_wait(r.ctx, 2000)
        assert st == L.XR_ERR_TIMEOUT, lib.xr_last_error(r.ctx)
        assert b"timed out" in lib.xr_last_error(r.ctx)
        assert r.stats().error_flags & L.XR_DEVFLAG_MMA_TIMEOUT
        assert lib.xr_cache_selftest_wait(r.ctx, 0) == L.XR_ERR_INVALID_ARGUMENT
        from tests.helpers import camera_sequence
        for u in camera_sequence(scene, 32, 32, 2, 4):
            r.render(u)                   # the context is still usable: the flag was seen once
        img = r.read_output(L.XR_OUT_LDR8)
        assert img.reshape(-1, 4)[:, :3].mean() > 1.0
