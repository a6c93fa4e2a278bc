"""The README's Scene1 -- Sibenik (asset/model/sb2, src/main.cpp:56-57; 75,277
triangles, base-colour textures, one emissive material) -- through the CUDA
pipeline against the oracle, at the reference's default camera (lookAt from
(0, 1, 3), 45 degrees, src/Asset/Scene.cpp:30): 192 x 108 frames (the 1080p view
at 1/100 of the pixels) with a moving camera, bit-exact in reference mode with the
reference's 10 bounces and in corrected mode with the benchmark settings.

The scene comes from oracle/refpin/scenes.py (converted from the reference
checkout into oracle/_ref/scenes); the tests skip where it is not present.
"""
import pytest

import xvk_ray_gb300 as xr
from tests.helpers import camera_sequence
from tests.test_gpu_frames import _compare_frame, _setup

pytestmark = pytest.mark.gpu


def _scene():
    from oracle.refpin import scenes
    try:
        return scenes.load("sibenik")
    except FileNotFoundError as e:
        pytest.skip(str(e))


@pytest.mark.parametrize("compat", [True, False])
def test_sibenik_frames_bit_exact(compat):
    scene = _scene()
    assert scene.n_triangles == 75277 and len(scene.textures) == 3
    W, H = 192, 108
    bounces = 10 if compat else 4
    p = (xr.params_reference if compat else xr.params_default)(W, H, write_hdr=1)

    def move(f, cam):
        cam.position[0] += 0.05
        cam.yaw_deg += 1.0

    r, o = _setup(scene, p)
    with r:
        for f, u in enumerate(camera_sequence(scene, W, H, 3, bounces, move=move)):
            r.render(u)
            o.render(u)
            _compare_frame(r, o, compat, f"frame {f}")
