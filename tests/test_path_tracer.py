"""The PathTracer render-pass interface (src/pathTracer.h:12-57) in both host
languages: the C++ header include/xr_path_tracer.hpp and the Python mirror
xvk_ray_gb300.path_tracer.  The C++ driver compiles and links against libxr.so
without a GPU; on the GPU both render the same Cornell frames bit for bit, and
the same frames as direct Renderer calls with the UBOs PathTracer builds."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import xvk_ray_gb300 as xr
from xvk_ray_gb300 import _build
from xvk_ray_gb300 import _lib as L

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "path_tracer_frames.cpp"


def _compile(out: Path) -> Path:
    lib = _build.LIB
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", f"-I{ROOT / 'include'}", str(SRC), "-o", str(out),
           f"-L{lib.parent}", "-lxr", f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "warning" not in r.stderr, r.stderr
    return out


def test_cpp_path_tracer_compiles_and_links(tmp_path):
    exe = _compile(tmp_path / "path_tracer_frames")
    # without arguments it prints its usage and exits 2 (no GPU needed)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def _python_frames(w, h, frames, compat):
    pt = xr.PathTracer(xr.UserSettings(compat_reference=compat), w, h)
    try:
        pt.PostTracerInit([xr.Scene.cornell()])
        ubos = []
        for _ in range(frames):
            pt.DrawFrame()
            ubos.append(pt._prev_ubo)
        return pt.renderer.read_output(L.XR_OUT_LDR8).copy(), ubos
    finally:
        pt.close()


@pytest.mark.gpu
@pytest.mark.parametrize("compat", [False, True])
def test_cpp_and_python_path_tracers_render_identical_frames(tmp_path, compat):
    w, h, frames = 64, 48, 4
    exe = _compile(tmp_path / "path_tracer_frames")
    out = tmp_path / "frame.rgba8"
    r = subprocess.run([str(exe), str(w), str(h), str(frames), str(out), "1" if compat else "0"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cpp = np.frombuffer(out.read_bytes(), np.uint8).reshape(h, w, 4)
    py, ubos = _python_frames(w, h, frames, compat)
    assert np.array_equal(cpp.reshape(-1), np.asarray(py).reshape(-1).view(np.uint8))
    # the same frames through Renderer calls with PathTracer's UBOs
    with xr.Renderer(w, h) as rd:
        rd.set_params(xr.params_reference(w, h) if compat else xr.params_default(w, h))
        rd.upload_scene(xr.Scene.cornell())
        rd.build_bvh()
        for f, u in enumerate(ubos):
            assert u.current_frame == f + 1   # DrawFrame advances the counter first (pathTracer.cpp:135)
            rd.render(u)
        assert np.array_equal(np.asarray(rd.read_output(L.XR_OUT_LDR8)).reshape(-1).view(np.uint8), cpp.reshape(-1))
    assert cpp[..., :3].max() > 0
