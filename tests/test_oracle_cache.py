"""CPU checks of the learned-radiance-cache oracle (oracle/nrc.cpp).

The reference renderer has no learned cache; the oracle restates the published
hash encoding (Mueller et al. 2022), the radiance-cache network and loss
(Mueller et al. 2021) and Adam (Kingma and Ba 2015).  It is pinned here by
central finite differences of its own loss in exact (FP64, unrounded) mode and
by an independent numpy restatement of the Adam step.
"""
import numpy as np
import pytest

from oracle import binding as ob


def _samples(rng, n):
    s = np.zeros(n, ob.CACHE_SAMPLE_DTYPE)
    s["pos"] = rng.uniform(-0.9, 0.9, (n, 3))
    nrm = rng.normal(size=(n, 3)); nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3)); wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    s["normal"], s["wo"] = nrm, wo
    s["albedo"] = rng.uniform(0, 1, (n, 3))
    s["roughness"] = rng.uniform(0.05, 1, n)
    s["kind"] = rng.choice([0, 1, 5], n)
    s["target"] = rng.uniform(0, 2, (n, 3))
    return s


@pytest.fixture(scope="module")
def cache():
    c = ob.OracleCache(seed=3)
    c.set_bounds([-1.0, -1.0, -1.0], 0.5)
    # larger table values than the 1e-4 initialisation so the grid path matters
    g = c.param(ob.NRC_GRID)
    g *= 2000.0
    yield c
    c.close()


def test_pack_roundtrip():
    rng = np.random.default_rng(0)
    s = _samples(rng, 64)
    rec = ob.pack_cache_samples(s)
    assert np.array_equal(rec[:, 0:3].view(np.float32), s["pos"])
    assert np.array_equal(rec[:, 7].view(np.float32), s["roughness"])
    assert np.array_equal(rec[:, 6] >> 24, s["kind"])
    assert np.array_equal(rec[:, 6] & 255, np.floor(s["albedo"][:, 0] * 255 + 0.5).astype(np.uint32))


def _fd_check(cache, arr, idx, rec, tgt, grad):
    bad = []
    for i in idx:
        w0 = arr[i]
        h = np.float32(max(abs(w0) * 2e-5, 1e-7))
        arr[i] = w0 + h; hp = np.float64(arr[i]); lp = cache.loss(rec, tgt, exact=True, loss_kind=1)
        arr[i] = w0 - h; hm = np.float64(arr[i]); lm = cache.loss(rec, tgt, exact=True, loss_kind=1)
        arr[i] = w0
        fd = (lp - lm) / (hp - hm)
        g = np.float64(grad[i])
        if abs(fd - g) > 2e-3 * max(abs(fd), abs(g)) + 1e-9:
            bad.append((int(i), fd, g))
    return bad


def test_gradients_match_finite_differences(cache):
    rng = np.random.default_rng(1)
    s = _samples(rng, 24)
    rec = ob.pack_cache_samples(s)
    tgt = s["target"]
    cache.backward(rec, tgt, exact=True, loss_kind=1)
    gw = cache.param(ob.NRC_MLP_GRAD).copy()
    gg = cache.param(ob.NRC_GRID_GRAD).copy()
    w = cache.param(ob.NRC_MLP)
    g = cache.param(ob.NRC_GRID)
    # MLP: 12 weights of each layer with a non-zero gradient
    idx = []
    for l in range(5):
        lo, hi = l * 4096, l * 4096 + (4096 if l < 4 else 1024)
        nz = lo + np.flatnonzero(gw[lo:hi])
        assert len(nz) > 12
        idx += list(rng.choice(nz, 12, replace=False))
    # a step can straddle a ReLU kink of one sample; at most one such parameter per set
    assert len(_fd_check(cache, w, idx, rec, tgt, gw)) <= 1
    # hash table: 40 touched values across the levels
    nz = np.flatnonzero(gg)
    assert len(nz) > 1000
    assert len(_fd_check(cache, g, rng.choice(nz, 40, replace=False), rec, tgt, gg)) <= 1


def test_gpu_mode_close_to_exact(cache):
    rng = np.random.default_rng(2)
    s = _samples(rng, 256)
    rec = ob.pack_cache_samples(s)
    a = cache.infer(rec, exact=False)
    b = cache.infer(rec, exact=True)
    rel = np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel < 3e-2


def test_adam_step_matches_numpy():
    c = ob.OracleCache(seed=5)
    try:
        rng = np.random.default_rng(4)
        w = c.param(ob.NRC_MLP); gw = c.param(ob.NRC_MLP_GRAD)
        g = c.param(ob.NRC_GRID); gg = c.param(ob.NRC_GRID_GRAD)
        w0, g0 = w.copy(), g.copy()
        gw[:] = rng.normal(size=gw.shape).astype(np.float32)
        touched = rng.choice(len(g), 1000, replace=False)
        gg[touched] = rng.normal(size=1000).astype(np.float32)
        lr, b1, b2, eps = np.float32(1e-2), np.float32(0.9), np.float32(0.99), np.float32(1e-15)
        bc1, bc2 = np.float32(1 - 0.9), np.float32(1 - 0.99)
        c.adam(lr, b1, b2, eps, bc1, bc2)

        def ref(p, grad):
            m = (b1 * np.float32(0) + (np.float32(1) - b1) * grad).astype(np.float32)
            v = (b2 * np.float32(0) + (np.float32(1) - b2) * (grad * grad)).astype(np.float32)
            return (p - lr * (m / bc1) / (np.sqrt(v / bc2) + eps)).astype(np.float32)

        assert np.array_equal(w, ref(w0, gw))
        assert np.array_equal(g[touched], ref(g0[touched], gg[touched]))
        untouched = np.setdiff1d(np.arange(0, len(g), 997), touched)
        assert np.array_equal(g[untouched], g0[untouched])
    finally:
        c.close()
