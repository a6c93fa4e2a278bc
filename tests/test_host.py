"""Host-side checks of libxr.so (no GPU work)."""
import ctypes as C
import math
import re
from pathlib import Path

import numpy as np
import pytest

import xvk_ray_gb300 as xr

L = xr._lib
ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_declared_symbol():
    header = (ROOT / "include" / "xr.h").read_text()
    declared = set(re.findall(r"\b(xr_[a-z0-9_]+)\s*\(", header))
    lib = C.CDLL(str(L.LIB_PATH))
    missing = [name for name in sorted(declared) if not hasattr(lib, name)]
    assert not missing, missing
    assert declared <= set(L.EXPORTED) | {"xr_api_version"}


def test_struct_layouts_match_the_reference():
    # AVertex 36 B, AMaterial 32 B, UniformBufferObject 412 B (src/Asset/*.h)
    assert C.sizeof(L.XrVertex) == 36
    assert C.sizeof(L.XrMaterial) == 32
    assert C.sizeof(L.XrUniformBufferObject) == 412
    assert C.sizeof(L.XrInstance) == 56   # {scene, reserved, 3 x 4 object-to-world}
    assert L.load().xr_api_version() == 1


def test_instance_records_pack_like_the_struct():
    """pack_instances gives the bytes a ctypes XrInstance array holds (matrices
    rounded to float the same way), and passes record arrays through unchanged."""
    rng = np.random.default_rng(4)
    pairs = [(int(k), rng.normal(size=(3, 4))) for k in rng.integers(0, 5, 9)]
    arr = xr.pack_instances(pairs)
    ref = (L.XrInstance * len(pairs))()
    for i, (k, m) in enumerate(pairs):
        ref[i].scene = k
        ref[i].object_to_world[:] = [float(x) for x in m.reshape(12)]
    assert arr.tobytes() == bytes(ref)
    assert xr.pack_instances(arr) is arr or np.array_equal(xr.pack_instances(arr), arr)
    assert xr.pack_instances([]).shape == (0,)


def test_no_silent_cpu_fallback():
    """Creating a context needs a CUDA device; without one the call fails loudly."""
    lib = L.load()
    n = C.c_int(0)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    st = lib.xr_create(C.byref(L.XrDeviceDesc(0, 64, 64)), C.byref(h))
    assert st == L.XR_ERR_CUDA and not h.value
    assert b"CUDA" in lib.xr_last_error(None) or b"device" in lib.xr_last_error(None)


def test_parameter_presets():
    d = xr.params_default(1920, 1080)
    assert (d.compat_reference, d.m_cap_temporal, d.n_neighbours, d.radius_px, d.visibility) == (0, 20, 5, 30.0, 1)
    r = xr.params_reference(1920, 1080)
    assert (r.compat_reference, r.m_cap_temporal, r.m_cap_spatial, r.n_neighbours, r.radius_px) == (1, 30, 300, 6, 5.0)


def test_cornell_scene():
    s = xr.Scene.cornell()
    assert s.n_triangles == 36 and s.materials.shape == (4, 8)
    model = s.materials[:, 7].view(np.uint32)
    light = np.where(model == L.XR_MAT_DIFFUSE_LIGHT)[0]
    assert len(light) == 1
    assert np.allclose(s.materials[light[0], :3] * 4.0, [17, 12, 4])     # emission = baseColor * 4
    assert np.allclose(np.linalg.norm(s.vertices[:, 3:6], axis=1), 1.0, atol=1e-6)
    assert np.all(s.global_indices() < s.vertices.shape[0])


def test_procedural_scene_is_deterministic_and_in_range():
    a = xr.Scene.procedural(seed=7, n_objects=256)
    b = xr.Scene.procedural(seed=7, n_objects=256)
    assert np.array_equal(a.vertices, b.vertices) and np.array_equal(a.indices, b.indices)
    m = a.materials
    model = m[:, 7].view(np.uint32)
    obj = (model == L.XR_MAT_METALLIC) | (model == L.XR_MAT_PLASTIC)
    assert obj.sum() == 256
    assert np.all((m[obj, 5] >= 0.05) & (m[obj, 5] <= 1.0))               # roughness U[0.05, 1]
    assert np.all((m[obj, :3] >= 0.1) & (m[obj, :3] <= 0.9))              # albedo U[0.1, 0.9]
    assert 0.15 < np.mean(model[obj] == L.XR_MAT_METALLIC) < 0.45          # Bernoulli(0.3)
    lights = model == L.XR_MAT_DIFFUSE_LIGHT
    assert np.all((m[lights, 0] * 4 >= 5) & (m[lights, 0] * 4 <= 50))      # radiance U[5, 50]


def test_full_size_procedural_scene_has_about_a_million_triangles():
    s = xr.Scene.procedural()
    assert 990_000 < s.n_triangles < 1_010_000


def test_camera_ubo_matches_glm_conventions():
    cam = L.XrCamera((0.5, 1.0, 3.0), 10.0, 5.0, 45.0)
    u = xr.camera_ubo(cam, 1920, 1080, None, 0, 4)
    view = np.array(u.view, np.float64).reshape(4, 4).T          # column-major -> row-major
    proj = np.array(u.projection, np.float64).reshape(4, 4).T
    th = math.tan(math.radians(45.0) / 2)
    assert math.isclose(proj[0, 0], 1 / ((1920 / 1080) * th), rel_tol=1e-6)
    assert math.isclose(proj[1, 1], -1 / th, rel_tol=1e-6)                  # projection[1][1] *= -1
    assert math.isclose(proj[3, 2], -1.0) and math.isclose(proj[2, 2], 1000 / (0.001 - 1000), rel_tol=1e-6)
    assert np.allclose(view @ np.array(u.view_inverse, np.float64).reshape(4, 4).T, np.eye(4), atol=1e-5)
    assert np.allclose(proj @ np.array(u.projection_inverse, np.float64).reshape(4, 4).T, np.eye(4), atol=1e-4)
    assert np.allclose(view @ [0.5, 1.0, 3.0, 1.0], [0, 0, 0, 1], atol=1e-6)   # camera at the origin
    u2 = xr.camera_ubo(cam, 1920, 1080, u, 1, 4)
    assert list(u2.view_prev) == list(u.view) and list(u.view_prev) == list(u.view)   # first frame: prev = current


def test_png_roundtrip(tmp_path):
    """Headless output (the reference's present path replaced by a PNG file)."""
    from xvk_ray_gb300.render import read_png_rgba, write_png
    rng = np.random.default_rng(3)
    for w, h in ((1, 1), (7, 3), (64, 48)):
        px = rng.integers(0, 256, (w * h, 4)).astype(np.uint8)
        p = tmp_path / f"i{w}x{h}.png"
        write_png(str(p), px, w, h)
        back, bw, bh = read_png_rgba(str(p))
        assert (bw, bh) == (w, h) and np.array_equal(back, px)


def test_workload_library_generates_the_benchmark_inputs():
    """oracle/_build/libworkload.so (the generator built without libxr.so, for the
    CPU baseline) yields the benchmark scene and camera path bit for bit."""
    from oracle import workload as wl
    kw = dict(seed=1, n_objects=64, n_lights=4, extent=8.0, sphere_subdiv=2)
    a, b = wl.procedural(**kw), xr.Scene.procedural(**kw)
    for k in ("vertices", "indices", "materials"):
        assert np.array_equal(getattr(a, k).view(np.uint32), getattr(b, k).view(np.uint32)), k
    assert bytes(a.camera) == bytes(b.camera)
    assert np.array_equal(wl.cornell().vertices.view(np.uint32), xr.Scene.cornell().vertices.view(np.uint32))
    cam = xr._lib.XrCamera.from_buffer_copy(a.camera)
    pa = pb = None
    for f in range(3):
        cam.position[2] -= 0.01
        cam.yaw_deg += 0.2
        ua, ub = wl.camera_ubo(cam, 1920, 1080, pa, f, 4), xr.camera_ubo(cam, 1920, 1080, pb, f, 4)
        assert xr.ubo_bytes(ua) == xr.ubo_bytes(ub)
        pa, pb = ua, ub
