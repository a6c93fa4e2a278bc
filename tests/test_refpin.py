"""The oracle against the reference's own shader source (CPU).

tests/golden/ref_*.npz hold values computed by shader/HLSL/random.hlsl and
shader/HLSL/ReSTIRGI/*.hlsl themselves, compiled as C++ by oracle/refpin
(tests/golden/make_ref_fixtures.py).  The oracle's reference mode must
reproduce them: every helper, the temporal and spatial passes on fixed
candidates, and whole frames -- every word of every sample and reservoir and the
RGBA8 image.  The one relaxation is the sign of a zero (tests.helpers.canon):
the reference's hit shader maps normals through its identity instance
transform, where the driver's evaluation order decides whether -0 stays -0.

When the reference checkout is present (not on the GPU machine) the pin is also
built and run live against the oracle on scenes the fixtures do not hold.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import xvk_ray_gb300 as xr
from oracle import binding as ob
from oracle import refpin
from tests.helpers import (RES_FIELDS, RES_INT_WORDS, RES_SAMPLE_FIELDS, SAMPLE_FIELDS, SAMPLE_INT_WORDS,
                           box_scene, camera_sequence, canon, canon_floats, field_digests, scene_digest)

GOLDEN = Path(__file__).resolve().parent / "golden"
XR = xr._lib
ALL_RES_FIELDS = {**RES_FIELDS, **RES_SAMPLE_FIELDS}


def load_fixture(name: str) -> dict:
    """A fixture's arrays, held in a dict (an NpzFile makes a new array on every
    access, whose data pointer would not outlive a ctypes call)."""
    with np.load(GOLDEN / name) as z:
        return {k: (lambda a: a if a.ndim == 0 else np.ascontiguousarray(a))(z[k]) for k in z.files}


@pytest.fixture(scope="module")
def units():
    return load_fixture("ref_units.npz")


def _same_floats(a, b):
    assert np.array_equal(canon_floats(a), canon_floats(b))


def test_rng_matches_reference_source(units):
    lib = ob.load()
    for (x, y, w, h, f), seed, nxt, flt in zip(units["rng_px"], units["rng_seed"], units["rng_next"],
                                               units["rng_float"]):
        assert lib.or_init_random_seed(int(x), int(y), int(w), int(f)) == int(seed)
        u, fl = ob.random_sequence(int(seed), nxt.size)
        assert np.array_equal(u, nxt)
        assert np.array_equal(fl.view(np.uint32), flt.view(np.uint32))


def test_sampling_helpers_match_reference_source(units):
    lib = ob.load()
    n = units["onb_n"].shape[0]
    onb = np.empty((n, 6), np.float32)
    lib.or_units_onb(units["onb_n"].ctypes.data, n, onb.ctypes.data)
    _same_floats(onb, units["onb_out"])
    hemi = np.empty((units["hemi_xi"].shape[0], 3), np.float32)
    lib.or_units_sample_hemisphere(units["hemi_xi"].ctypes.data, hemi.shape[0], hemi.ctypes.data)
    _same_floats(hemi, units["hemi_out"])
    nb = units["bsdf_n"].shape[0]
    out = np.empty((nb, 9), np.float32)
    lib.or_units_sample_bsdf(*(units[k].ctypes.data for k in ("bsdf_n", "bsdf_wo", "bsdf_mat",
                                                                                    "bsdf_seed")), nb, out.ctypes.data)
    _same_floats(out, units["bsdf_out"])
    w2s = np.empty_like(units["w2s_out"])
    lib.or_units_world_to_screen_uv(units["w2s_p"].ctypes.data, w2s.shape[0],
                                    units["w2s_view"].ctypes.data,
                                    units["w2s_proj"].ctypes.data, w2s.ctypes.data)
    _same_floats(w2s, units["w2s_out"])
    aces = np.empty_like(units["aces_out"])
    lib.or_units_aces(units["aces_in"].ctypes.data, aces.shape[0], aces.ctypes.data)
    _same_floats(aces, units["aces_out"])


def test_reservoir_helpers_match_reference_source(units):
    lib = ob.load()
    nl = units["upd_seed"].size
    k = units["upd_w"].size // nl
    out = np.empty((nl, 28), np.uint32)
    so = np.empty(nl, np.uint32)
    lib.or_units_update_list(*(units[x].ctypes.data for x in ("upd_samples", "upd_w")), nl, k,
                             units["upd_seed"].ctypes.data, out.ctypes.data, so.ctypes.data)
    assert np.array_equal(canon(out, RES_INT_WORDS), canon(units["upd_out"], RES_INT_WORDS))
    assert np.array_equal(so, units["upd_seed_out"])
    lib.or_units_merge_list(*(units[x].ctypes.data for x in ("mrg_res", "mrg_phat")), nl, k,
                            units["mrg_seed"].ctypes.data, out.ctypes.data, so.ctypes.data)
    assert np.array_equal(canon(out, RES_INT_WORDS), canon(units["mrg_out"], RES_INT_WORDS))
    assert np.array_equal(so, units["mrg_seed_out"])
    n = units["sim_a"].shape[0]
    sim = np.empty((n, 2), np.uint32)
    lib.or_units_similar(units["sim_a"].ctypes.data,
                         units["sim_b"].ctypes.data, n, sim.ctypes.data)
    assert np.array_equal(sim, units["sim_out"])
    assert 0.2 < units["sim_out"][:, 0].mean() < 0.8          # both outcomes are exercised
    tg = np.empty((units["tgt_x"].shape[0], 2), np.float32)
    lib.or_units_targets(*(units[x].ctypes.data for x in ("tgt_samples", "tgt_x", "tgt_n")),
                         tg.shape[0], tg.ctypes.data)
    _same_floats(tg, units["tgt_out"])
    for (x, y, w, h, seed), r, row in zip(units["nb_case"], units["nb_radius"], units["nb_out"]):
        got = np.empty(6, np.uint32)
        lib.or_units_neighbor_index(int(x), int(y), int(w), int(h), float(r), int(seed), 6, got.ctypes.data)
        assert np.array_equal(got, row)


# ---------------------------------------------------------------------------
# passes on fixed candidates
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("case", ["kat", "surface"])
def test_fixed_candidate_passes_match_reference_source(case):
    g = load_fixture("ref_passes.npz")
    W, H = int(g[f"{case}_width"]), int(g[f"{case}_height"])
    ubo = XR.XrUniformBufferObject.from_buffer_copy(g[f"{case}_ubo"].tobytes())
    scene = xr.Scene.cornell()
    o = ob.OracleRenderer(ob.OracleScene.from_scene(scene), xr.params_reference(W, H))
    o.set_samples(g[f"{case}_samples"], ubo)
    o.write_temporal(g[f"{case}_temporal_in"])
    ubo.reuse = 0
    o.run_pass(ubo, 1)
    assert np.array_equal(canon(o.read(ob.BUF_TEMPORAL), RES_INT_WORDS),
                          canon(g[f"{case}_temporal_out"], RES_INT_WORDS))
    assert np.array_equal(canon(o.read(ob.BUF_SPATIAL), RES_INT_WORDS),
                          canon(g[f"{case}_spatial_after_temporal"], RES_INT_WORDS))
    ldr = o.read(ob.BUF_LDR).reshape(-1, 4)[:, :3]
    assert np.array_equal(ldr, g[f"{case}_ldr_temporal"][:, :3])
    merged = 0
    for reuse in (1, 0):
        ubo.reuse = reuse
        o.run_pass(ubo, 2)
        sp = o.read(ob.BUF_SPATIAL)
        assert np.array_equal(canon(sp, RES_INT_WORDS), canon(g[f"{case}_spatial_out_reuse{reuse}"], RES_INT_WORDS))
        assert np.array_equal(o.read(ob.BUF_LDR).reshape(-1, 4)[:, :3], g[f"{case}_ldr_reuse{reuse}"][:, :3])
        merged = max(merged, int(sp[:, 2].max()))
    if case == "surface":
        # neighbours passed the similarity test and were merged (M beyond one reservoir's)
        assert merged > 30


def test_python_restatement_agrees_with_reference_source():
    """temporal_kat.npz (from the independent Python restatement tests/pyref.py)
    against the reference source's own temporal pass on the same candidates."""
    kat = load_fixture("temporal_kat.npz")
    g = load_fixture("ref_passes.npz")
    for k, sl in RES_FIELDS.items():
        a = canon(kat["temporal_out"], RES_INT_WORDS)[:, sl]
        b = canon(g["kat_temporal_out"], RES_INT_WORDS)[:, sl]
        assert np.array_equal(a, b), k


# ---------------------------------------------------------------------------
# whole frames
# ---------------------------------------------------------------------------
def frame_scene(g, key, name=None) -> "xr.Scene":
    """A sequence's scene: stored in the fixture, or (`ext:<name>`) one of the
    reference's glTF scenes converted by oracle/refpin/scenes.py, checked against
    the SHA-1 the fixture recorded; skips when that scene is not available."""
    if key.startswith("ext:"):
        from oracle.refpin import scenes
        try:
            sc = scenes.load(key[4:])
        except FileNotFoundError as e:
            pytest.skip(str(e))
        assert scene_digest(sc) == str(g[f"{name}_scene_sha1"]), "converted scene differs from the fixture's"
        return sc
    cam = XR.XrCamera.from_buffer_copy(g[f"scene_{key}_camera"].tobytes())
    tex = [g[f"scene_{key}_texture{t}"] for t in range(int(g[f"scene_{key}_ntex"]))]
    return xr.Scene(g[f"scene_{key}_vertices"], g[f"scene_{key}_indices"], g[f"scene_{key}_materials"],
                    g[f"scene_{key}_ranges"], cam, tex)


def frame_sequences():
    return json.loads(str(load_fixture("ref_frames.npz")["sequences"]))


def frame_digests(samples, temporal, spatial, res_fields=ALL_RES_FIELDS) -> dict:
    d = {"samples." + k: v for k, v in field_digests(samples, SAMPLE_FIELDS, SAMPLE_INT_WORDS).items()}
    d.update({"temporal." + k: v for k, v in field_digests(temporal, res_fields, RES_INT_WORDS).items()})
    d.update({"spatial." + k: v for k, v in field_digests(spatial, res_fields, RES_INT_WORDS).items()})
    return d


@pytest.mark.parametrize("name", frame_sequences())
def test_frames_match_reference_source(name):
    g = load_fixture("ref_frames.npz")
    meta = json.loads(str(g[f"{name}_meta"]))
    scene = frame_scene(g, meta["scene"], name)
    W, H = meta["width"], meta["height"]
    o = ob.OracleRenderer(ob.OracleScene.from_scene(scene), xr.params_reference(W, H))
    digests = json.loads(str(g[f"{name}_digests"]))
    for f, (ub, want) in enumerate(zip(g[f"{name}_ubos"], digests)):
        o.render(XR.XrUniformBufferObject.from_buffer_copy(ub.tobytes()))
        got = frame_digests(o.read(ob.BUF_SAMPLES), o.read(ob.BUF_TEMPORAL), o.read(ob.BUF_SPATIAL))
        bad = sorted(k for k in want if got[k] != want[k])
        assert not bad, f"frame {f}: {bad}"
        ldr = o.read(ob.BUF_LDR).reshape(-1, 4)[:, :3]
        assert np.array_equal(ldr, g[f"{name}_ldr"][f][:, :3]), f"frame {f}: image"


# ---------------------------------------------------------------------------
# the recipe itself
# ---------------------------------------------------------------------------
def test_rewrite_is_mechanical():
    src = ("float3 f(inout uint seed, out float3 b, in float2 xi : SV_Position)\n"
           "{ // comment 1.5\n b = float3(RandomFloat(seed), 2.0, x.xyz.x); return v.rgb * 0.5f + 1e-6; }\n"
           "cbuffer U : register(b3) { UBO u; };\n[shader(\"miss\")]\nTexture2D T[] : register(t8);\n")
    out = refpin.rewrite(src)
    assert "float3& b" in out and "uint& seed" in out and "float2 xi)" in out
    assert "float3{RandomFloat(seed), HLSL_LIT(2.0), x.xyz().x}" in out
    assert "v.rgb() * 0.5f + HLSL_LIT(1e-6)" in out
    assert "cbuffer" not in out and "register" not in out and "shader" not in out and "comment" not in out
    assert "UBO u;" in out and "Texture2D T[hlsl::kMaxTextures];" in out


def _live():
    if not refpin.available():
        pytest.skip("reference checkout not present")
    refpin.build()


@pytest.mark.parametrize("reuse", [True, False])
def test_live_oracle_matches_reference_source(reuse):
    """Built from the checkout on this machine: a box scene of 40 boxes and a light
    (Lambertian, the reference's material models), 40 x 30, camera moving, 6 bounces."""
    _live()
    scene = box_scene(np.random.default_rng(11), 40, 3.0)
    W, H = 40, 30

    def move(f, cam):
        cam.position[0] += 0.05
        cam.yaw_deg += 1.0

    ubos = camera_sequence(scene, W, H, 4, 6, move=move, reuse=reuse)
    rr = refpin.RefRenderer(refpin.RefScene(scene), W, H)
    o = ob.OracleRenderer(ob.OracleScene.from_scene(scene), xr.params_reference(W, H))
    for f, u in enumerate(ubos):
        rr.render(u)
        o.render(u)
        want = frame_digests(rr.read(refpin.BUF_SAMPLES), rr.read(refpin.BUF_TEMPORAL), rr.read(refpin.BUF_SPATIAL))
        got = frame_digests(o.read(ob.BUF_SAMPLES), o.read(ob.BUF_TEMPORAL), o.read(ob.BUF_SPATIAL))
        assert sorted(k for k in want if got[k] != want[k]) == [], f"frame {f}"
        from tests.helpers import unorm8
        assert np.array_equal(o.read(ob.BUF_LDR).reshape(-1, 4)[:, :3], unorm8(rr.read(refpin.BUF_OUTPUT))[:, :3])
        assert np.array_equal(canon_floats(o.read(ob.BUF_GBUF_POS).reshape(-1, 4)),
                              canon_floats(rr.read(refpin.BUF_GPOS)))
        assert np.array_equal(canon_floats(o.read(ob.BUF_MOTION).reshape(-1, 2)),
                              canon_floats(rr.read(refpin.BUF_MOTION)))
