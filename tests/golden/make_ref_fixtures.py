"""Generates the reference-source fixtures tests/golden/ref_*.npz (run from the
repo root, where the reference checkout is present).

Every expected value below is computed by the reference's own shader code --
shader/HLSL/random.hlsl and shader/HLSL/ReSTIRGI/*.hlsl compiled as C++ by the
recipe in oracle/refpin (mechanical rewrite, HLSL shim, the reference's pipeline
wiring; traversal by the oracle, which the reference leaves to RT cores):

  ref_units.npz    the helpers one by one: InitRandomSeed / NextRandom /
                   RandomFloat, BranchlessONB, SampleHemisphere, SampleBSDF
                   (Lambertian, DiffuseLight, other models), UpdateReservoir and
                   MergeReservoir on fixed candidate lists, both IsSimilar
                   overloads, ACESFilm, EvaluateTargetFunction and p_hat,
                   WorldToScreenUV, GetNeighborIndex
  ref_passes.npz   the temporal and spatial passes (reference mode) on fixed
                   candidates: the 8x8 hand-built candidates of temporal_kat.npz,
                   and a 16x16 hand-built surface whose neighbours pass the
                   similarity test (Jacobian, M arithmetic, merges)
  ref_frames.npz   whole reference-mode frames (ApplicationReSTIRGI::Render):
                   per frame the SHA-1 of every sample and reservoir field and the
                   RGBA8 image, for Cornell-box sequences (static and moving camera,
                   reuse on and off, textured with sky, two models with 8 bounces)

Scenes and UBOs are stored in the fixtures, so the tests need neither the
reference nor the host code that generated them.  The SHA-256 of each shader
file used is recorded as `shader_sha256`.
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import xvk_ray_gb300 as xr  # noqa: E402
from oracle import refpin  # noqa: E402
from tests.helpers import (RES_FIELDS, RES_INT_WORDS, RES_SAMPLE_FIELDS, SAMPLE_FIELDS,  # noqa: E402
                           SAMPLE_INT_WORDS, box_scene, camera_sequence, field_digests, scene_digest, unorm8)

HERE = Path(__file__).resolve().parent
C = xr._lib
ALL_RES_FIELDS = {**RES_FIELDS, **RES_SAMPLE_FIELDS}


def shader_hashes() -> str:
    src = refpin.REFERENCE_ROOT / "shader" / "HLSL"
    return json.dumps({rel: hashlib.sha256((src / rel).read_bytes()).hexdigest() for rel in refpin.SHADERS})


# ---------------------------------------------------------------------------
# helpers one by one
# ---------------------------------------------------------------------------
def _unit_normals(rng, n):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    v = v.astype(np.float32)
    v[:8] = [[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, 1, 0], [0, 0, 0], [0, 0, -0.0],
             [1e-4, 0, -0.99999999], [-0.6, 0.8, 0]]
    return v


def _samples(rng, n):
    """Random ReSTIRGISample records (24 words)."""
    w = np.zeros((n, 24), np.uint32)
    f = w.view(np.float32)
    f[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    w[:, 3] = rng.integers(0, 4, n)
    f[:, 4:7] = _unit_normals(rng, n)
    w[:, 7] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    f[:, 8:11] = rng.uniform(-2, 2, (n, 3))
    f[:, 11] = rng.uniform(0, 0.4, n)
    f[:, 12:15] = _unit_normals(rng, n)
    f[:, 16:19] = rng.uniform(0, 5, (n, 3)) * (rng.random((n, 1)) > 0.1)
    f[:, 20:23] = rng.uniform(0, 0.3, (n, 3))
    return w


def units():
    lib = refpin.load()
    rng = np.random.default_rng(20261204)
    out = {}
    # RNG
    px = np.array([(0, 0, 1920, 1080, 0), (1, 0, 1920, 1080, 0), (1919, 1079, 1920, 1080, 9999),
                   (37, 11, 256, 256, 3), (255, 255, 256, 256, 7), (5, 5, 7, 3, 4294967294)] +
                  [tuple(int(v) for v in (rng.integers(0, 64), rng.integers(0, 48), 64, 48, rng.integers(0, 1000)))
                   for _ in range(26)], np.uint32)
    out["rng_px"] = px
    out["rng_seed"] = np.array([lib.ref_init_random_seed(*map(int, r)) for r in px], np.uint32)
    seqs_u, seqs_f = [], []
    for s in out["rng_seed"]:
        u = np.empty(32, np.uint32); f = np.empty(32, np.float32)
        sn = np.empty(32, np.float32); d = np.empty(64, np.float32)
        lib.ref_random_sequence(int(s), 32, u.ctypes.data, f.ctypes.data, sn.ctypes.data, d.ctypes.data)
        seqs_u.append(u); seqs_f.append(f)
    out["rng_next"], out["rng_float"] = np.stack(seqs_u), np.stack(seqs_f)
    # ONB, hemisphere
    n = 256
    out["onb_n"] = _unit_normals(rng, n)
    out["onb_out"] = np.empty((n, 6), np.float32)
    lib.ref_onb(out["onb_n"].ctypes.data, n, out["onb_out"].ctypes.data)
    xi = rng.random((n, 2)).astype(np.float32)
    xi[:4] = [[0, 0], [0.99999994, 0.99999994], [0.5, 0], [0.25, 0.99999994]]
    out["hemi_xi"] = xi
    out["hemi_out"] = np.empty((n, 3), np.float32)
    lib.ref_sample_hemisphere(xi.ctypes.data, n, out["hemi_out"].ctypes.data)
    # SampleBSDF
    mats = np.zeros((n, 8), np.float32)
    mats[:, 0:3] = rng.uniform(0, 1, (n, 3))
    mats[:, 3] = 1.0
    mats[:, 4] = np.full(n, -1, np.int32).view(np.float32)
    mats[:, 7] = rng.choice(np.array([0, 0, 0, 4, 1, 2], np.uint32), n).view(np.float32)
    out["bsdf_n"] = _unit_normals(rng, n)
    out["bsdf_wo"] = _unit_normals(rng, n)
    out["bsdf_mat"] = mats.view(np.uint32)
    out["bsdf_seed"] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    out["bsdf_out"] = np.empty((n, 9), np.float32)
    lib.ref_sample_bsdf(out["bsdf_n"].ctypes.data, out["bsdf_wo"].ctypes.data, out["bsdf_mat"].ctypes.data,
                        out["bsdf_seed"].ctypes.data, n, out["bsdf_out"].ctypes.data)
    # UpdateReservoir lists
    nl, k = 96, 6
    out["upd_samples"] = _samples(rng, nl * k)
    w = rng.uniform(0, 3, nl * k).astype(np.float32)
    w[rng.random(nl * k) < 0.2] = 0.0
    w[rng.random(nl * k) < 0.05] = np.float32(1e-12)
    w[rng.random(nl * k) < 0.05] = np.float32(1e6)
    out["upd_w"] = w
    out["upd_seed"] = rng.integers(0, 2**32, nl, dtype=np.uint64).astype(np.uint32)
    out["upd_out"] = np.empty((nl, 28), np.uint32)
    out["upd_seed_out"] = np.empty(nl, np.uint32)
    lib.ref_update_list(out["upd_samples"].ctypes.data, w.ctypes.data, nl, k, out["upd_seed"].ctypes.data,
                        out["upd_out"].ctypes.data, out["upd_seed_out"].ctypes.data)
    # MergeReservoir lists
    res = np.zeros((nl * k, 28), np.uint32)
    rf = res.view(np.float32)
    rf[:, 0] = rng.uniform(0, 10, nl * k)
    rf[:, 1] = rng.uniform(0, 3, nl * k) * (rng.random(nl * k) > 0.15)
    res[:, 2] = rng.integers(0, 40, nl * k)
    res[:, 4:28] = _samples(rng, nl * k)
    out["mrg_res"] = res
    ph = rng.uniform(0, 4, nl * k).astype(np.float32)
    ph[rng.random(nl * k) < 0.2] = 0.0
    out["mrg_phat"] = ph
    out["mrg_seed"] = rng.integers(0, 2**32, nl, dtype=np.uint64).astype(np.uint32)
    out["mrg_out"] = np.empty((nl, 28), np.uint32)
    out["mrg_seed_out"] = np.empty(nl, np.uint32)
    lib.ref_merge_list(res.ctypes.data, ph.ctypes.data, nl, k, out["mrg_seed"].ctypes.data,
                       out["mrg_out"].ctypes.data, out["mrg_seed_out"].ctypes.data)
    # IsSimilar: pairs near each threshold
    a = _samples(rng, n)
    b = a.copy()
    bf, af = b.view(np.float32), a.view(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dist = np.sqrt(rng.uniform(0.05, 0.15, n))      # |dx|^2 around 0.1
    bf[:, 0:3] = af[:, 0:3] + (d * dist[:, None]).astype(np.float32)
    tilt = rng.uniform(0.5, 0.8, n)                  # n.n' around 0.8
    t = _unit_normals(rng, n)
    nn = af[:, 4:7] * np.cos(tilt)[:, None] + t * np.sin(tilt)[:, None]
    with np.errstate(invalid="ignore"):       # the zero normals of _unit_normals give NaN pairs: kept as edge cases
        bf[:, 4:7] = (nn / np.linalg.norm(nn, axis=1, keepdims=True)).astype(np.float32)
    b[:, 3] = np.where(rng.random(n) < 0.8, a[:, 3], a[:, 3] + 1)
    out["sim_a"], out["sim_b"] = a, b
    out["sim_out"] = np.empty((n, 2), np.uint32)
    lib.ref_similar(a.ctypes.data, b.ctypes.data, n, out["sim_out"].ctypes.data)
    # ACESFilm
    c = rng.uniform(-0.5, 20, (n, 3)).astype(np.float32)
    c[:3] = [[0, 0, 0], [1, 1, 1], [1e6, 0.5, -1]]
    out["aces_in"] = c
    out["aces_out"] = np.empty((n, 3), np.float32)
    lib.ref_aces(c.ctypes.data, n, out["aces_out"].ctypes.data)
    # temporal EvaluateTargetFunction (ReSTIRGITemporalReuse.rgen.hlsl:33-40) and p_hat
    ts = _samples(rng, n)
    x = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    nrm = _unit_normals(rng, n)
    out["tgt_samples"], out["tgt_x"], out["tgt_n"] = ts, x, nrm
    tgt = np.empty((n, 2), np.float32)
    lib.ref_eval_target(ts.ctypes.data, x.ctypes.data, nrm.ctypes.data, n, tgt.ctypes.data)
    out["tgt_out"] = tgt
    # WorldToScreenUV with a camera's previous matrices
    scene = xr.Scene.cornell()
    u = camera_sequence(scene, 64, 48, 2, 4, move=lambda f, cam: setattr(cam, "yaw_deg", cam.yaw_deg + 3.0))[1]
    pts = rng.uniform([-1, 0, -1], [1, 2, 1], (n, 3)).astype(np.float32)
    out["w2s_p"] = pts
    out["w2s_view"] = np.array(u.view_prev, np.float32)
    out["w2s_proj"] = np.array(u.projection_prev, np.float32)
    out["w2s_out"] = np.empty((n, 2), np.float32)
    lib.ref_world_to_screen_uv(pts.ctypes.data, n, out["w2s_view"].ctypes.data, out["w2s_proj"].ctypes.data,
                               out["w2s_out"].ctypes.data)
    # GetNeighborIndex (ReSTIRGISpatialReuse.rgen.hlsl:35-42), borders included
    cases = []
    for i in range(128):
        x0 = int(rng.integers(0, 64)) if i % 4 else int(rng.choice([0, 63]))
        y0 = int(rng.integers(0, 48)) if i % 3 else int(rng.choice([0, 47]))
        cases.append((x0, y0, 64, 48, [5.0, 30.0][i % 2], int(rng.integers(0, 2**32, dtype=np.uint64))))
    out["nb_case"] = np.array([c[:4] + (c[5],) for c in cases], np.uint32)
    out["nb_radius"] = np.array([c[4] for c in cases], np.float32)
    nb = np.empty((128, 6), np.uint32)
    for i, c in enumerate(cases):
        row = np.empty(6, np.uint32)
        lib.ref_neighbor_index(c[0], c[1], c[2], c[3], c[4], c[5], 6, row.ctypes.data)
        nb[i] = row
    out["nb_out"] = nb
    out["shader_sha256"] = np.array(shader_hashes())
    np.savez_compressed(HERE / "ref_units.npz", **out)


# ---------------------------------------------------------------------------
# passes on fixed candidates
# ---------------------------------------------------------------------------
def _surface_case(rng, W=16, H=16):
    """A gently curved surface seen head on: neighbours within a few pixels are
    similar (|dx|^2 <= 0.1, n.n' >= 0.8, same material), so the spatial pass's
    Jacobian and merges run for most of them.  Materials are the Cornell box's
    Lambertian ones (the scene the passes run with)."""
    n = W * H
    s = np.zeros((n, 24), np.uint32)
    f = s.view(np.float32)
    yy, xx = np.mgrid[0:H, 0:W]
    u, v = xx.reshape(-1) / W, yy.reshape(-1) / H
    f[:, 0] = (u - 0.5) * 0.8
    f[:, 1] = 0.05 * np.sin(6 * u) * np.cos(5 * v)
    f[:, 2] = (v - 0.5) * 0.8
    nrm = np.stack([-0.3 * np.cos(6 * u) * np.cos(5 * v), np.ones(n), 0.25 * np.sin(6 * u) * np.sin(5 * v)], 1)
    f[:, 4:7] = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    s[:, 3] = np.where(rng.random(n) < 0.9, 1, 2)
    s[:, 7] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    f[:, 8:11] = rng.uniform([-1.5, 0.2, -1.5], [1.5, 2.0, 1.5], (n, 3))
    f[:, 11] = rng.uniform(0.02, 0.32, n)
    ns = rng.normal(size=(n, 3))
    ns[:, 1] -= 1.0                                   # sample normals mostly face the surface
    f[:, 12:15] = ns / np.linalg.norm(ns, axis=1, keepdims=True)
    f[:, 16:19] = rng.uniform(0, 3, (n, 3))
    # f of a Lambertian visible point is its material's albedo / pi (BSDF.hlsl:22-24)
    albedo = xr.Scene.cornell().materials[:, :3]
    f[:, 20:23] = albedo[s[:, 3]] * np.float32(1.0 / 3.14159265359)
    hole = rng.random(n) < 0.05                      # a few misses and lights
    s[hole] = 0
    s[hole, 3] = 0xFFFFFFFF
    light = (~hole) & (rng.random(n) < 0.05)
    f[light, 12:15] = 0.0
    temporal = np.zeros((2 * n, 28), np.uint32)
    tf = temporal.view(np.float32)
    src = rng.integers(0, n, 2 * n)
    temporal[:, 4:28] = s[src]
    tf[:, 0] = rng.uniform(0, 8, 2 * n)
    tf[:, 1] = rng.uniform(0, 2, 2 * n) * (rng.random(2 * n) > 0.1)
    temporal[:, 2] = rng.integers(1, 31, 2 * n)
    return W, H, s, temporal


def passes():
    kat = np.load(HERE / "temporal_kat.npz")
    rng = np.random.default_rng(77)
    cases = [("kat", int(kat["width"]), int(kat["height"]), kat["samples"], kat["temporal_in"], kat["ubo"])]
    W, H, s, t = _surface_case(rng)
    scene = xr.Scene.cornell()
    u0 = camera_sequence(scene, W, H, 1, 4)[0]
    cam = C.XrCamera.from_buffer_copy(scene.camera)
    cam.position[0] += 0.02
    u1 = xr.camera_ubo(cam, W, H, u0, 7, 4, reuse=False)
    cases.append(("surface", W, H, s, t, np.frombuffer(xr.ubo_bytes(u1), np.uint8)))
    out = {"cases": np.array([c[0] for c in cases])}
    rs = refpin.RefScene(scene)   # the passes trace only the spatial pass's no-op visibility rays
    for name, W, H, samples, temporal, ubo_bytes in cases:
        ubo = C.XrUniformBufferObject.from_buffer_copy(np.asarray(ubo_bytes, np.uint8).tobytes())
        rr = refpin.RefRenderer(rs, W, H)
        rr.set_gbuffer_from_samples(ubo, samples)
        ubo.reuse = 0
        rr.run_pass(ubo, 1, samples, temporal)
        t_out, s_after_t = rr.read(refpin.BUF_TEMPORAL), rr.read(refpin.BUF_SPATIAL)
        img_t = unorm8(rr.read(refpin.BUF_OUTPUT))
        for reuse in (1, 0):
            ubo.reuse = reuse
            rr.run_pass(ubo, 2)
            out[f"{name}_spatial_out_reuse{reuse}"] = rr.read(refpin.BUF_SPATIAL)
            out[f"{name}_ldr_reuse{reuse}"] = unorm8(rr.read(refpin.BUF_OUTPUT))
        out.update({f"{name}_width": W, f"{name}_height": H, f"{name}_samples": samples,
                    f"{name}_temporal_in": temporal, f"{name}_ubo": np.asarray(ubo_bytes, np.uint8),
                    f"{name}_temporal_out": t_out, f"{name}_spatial_after_temporal": s_after_t,
                    f"{name}_ldr_temporal": img_t})
        rr.close()
    out["shader_sha256"] = np.array(shader_hashes())
    np.savez_compressed(HERE / "ref_passes.npz", **out)


# ---------------------------------------------------------------------------
# whole frames
# ---------------------------------------------------------------------------
def textured_cornell():
    s = xr.Scene.cornell()
    rng = np.random.default_rng(4)
    tex = [rng.integers(0, 256, (5, 7, 4)).astype(np.uint8), rng.integers(64, 256, (16, 3, 4)).astype(np.uint8)]
    v = s.vertices.copy()
    v[:, 6] = v[:, 0] * 0.7 + v[:, 2] * 0.3 + 0.5
    v[:, 7] = v[:, 1] * 0.9 - 0.2
    m = s.materials.copy()
    models = m[:, 7].view(np.uint32)
    for k in range(m.shape[0]):
        if models[k] == 0:
            m[k, 4] = np.array([k % 2], np.int32).view(np.float32)[0]
        elif models[k] == 4:
            m[k, 4] = np.array([1], np.int32).view(np.float32)[0]
    return xr.Scene(v, s.indices, m, s.ranges, s.camera, tex)


def two_models():
    """The Cornell box and a box scene as two models (two ranges, model-local indices)."""
    a = xr.Scene.cornell()
    b = box_scene(np.random.default_rng(3), 6, 0.6, light=False)
    bv = b.vertices.copy()
    bv[:, 0:3] = bv[:, 0:3] * 0.5 + np.array([0.2, 0.4, 0.1], np.float32)
    mi = bv[:, 8].view(np.int32).copy()
    mi += a.materials.shape[0]
    bv[:, 8] = mi.view(np.float32)
    v = np.concatenate([a.vertices, bv])
    i = np.concatenate([a.indices, b.indices]).astype(np.uint32)
    m = np.concatenate([a.materials, b.materials[:2]])
    ranges = np.array([[0, 0], [a.indices.size, a.vertices.shape[0]]], np.uint32)
    return xr.Scene(v, i, m, ranges, a.camera)


def _move_after(k):
    def move(f, cam):
        if f >= k:
            cam.position[0] += 0.02
            cam.yaw_deg += 0.5
    return move


SEQUENCES = [
    # name, scene, W, H, frames, bounces, camera move, sky, reuse
    ("cornell_reuse", "cornell", 64, 48, 6, 4, 3, False, True),
    ("cornell_noreuse", "cornell", 64, 48, 3, 4, 1, False, False),
    ("textured_sky", "textured", 48, 40, 3, 4, 0, True, True),
    ("two_models_8_bounces", "two_models", 48, 40, 3, 8, 1, False, True),
    # the README's Scene1 (asset/model/sb2) with the reference's own settings (10 bounces, its
    # default camera): the scene is not stored here, only its SHA-1 (oracle/refpin/scenes.py)
    ("sibenik_reference_settings", "ext:sibenik", 96, 54, 3, 10, 1, False, True),
]


def frames():
    scenes = {"cornell": xr.Scene.cornell(), "textured": textured_cornell(), "two_models": two_models()}
    out = {"sequences": np.array(json.dumps([s[0] for s in SEQUENCES]))}
    for key, sc in scenes.items():
        out[f"scene_{key}_vertices"] = sc.vertices
        out[f"scene_{key}_indices"] = sc.indices
        out[f"scene_{key}_materials"] = sc.materials
        out[f"scene_{key}_ranges"] = sc.ranges
        out[f"scene_{key}_camera"] = np.frombuffer(bytes(sc.camera), np.uint8)
        for t, tex in enumerate(sc.textures):
            out[f"scene_{key}_texture{t}"] = tex
        out[f"scene_{key}_ntex"] = len(sc.textures)
    from oracle.refpin import scenes as ref_scenes
    for name, key, W, H, nf, bounces, move_at, sky, reuse in SEQUENCES:
        if key.startswith("ext:"):
            sc = ref_scenes.load(key[4:])
            out[f"{name}_scene_sha1"] = np.array(scene_digest(sc))
        else:
            sc = scenes[key]
        ubos = camera_sequence(sc, W, H, nf, bounces, move=_move_after(move_at), sky=sky, reuse=reuse)
        rs = refpin.RefScene(sc)
        rr = refpin.RefRenderer(rs, W, H)
        dig, ldr = [], []
        for u in ubos:
            rr.render(u)
            d = {"samples." + k: v for k, v in field_digests(rr.read(refpin.BUF_SAMPLES), SAMPLE_FIELDS,
                                                              SAMPLE_INT_WORDS).items()}
            for buf, label in ((refpin.BUF_TEMPORAL, "temporal"), (refpin.BUF_SPATIAL, "spatial")):
                d.update({f"{label}.{k}": v for k, v in field_digests(rr.read(buf), ALL_RES_FIELDS,
                                                                       RES_INT_WORDS).items()})
            dig.append(d)
            ldr.append(unorm8(rr.read(refpin.BUF_OUTPUT)))
        out[f"{name}_meta"] = np.array(json.dumps({"scene": key, "width": W, "height": H, "frames": nf,
                                                   "bounces": bounces, "sky": sky, "reuse": reuse}))
        out[f"{name}_ubos"] = np.stack([np.frombuffer(xr.ubo_bytes(u), np.uint8) for u in ubos])
        out[f"{name}_digests"] = np.array(json.dumps(dig))
        out[f"{name}_ldr"] = np.stack(ldr)
        rr.close()
        rs.close()
    out["shader_sha256"] = np.array(shader_hashes())
    np.savez_compressed(HERE / "ref_frames.npz", **out)


if __name__ == "__main__":
    from xvk_ray_gb300 import _build
    _build.build_library()
    _build.build_oracle()
    refpin.build()
    units()
    passes()
    frames()
    print("reference-source fixtures written to", HERE)
