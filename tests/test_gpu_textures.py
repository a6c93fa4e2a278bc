"""Base-colour textures (bilinear, clamp to edge, UNORM) and glTF scenes on the
GPU against the oracle: every sample, reservoir and the image bit-identical."""
import numpy as np
import pytest

import xvk_ray_gb300 as xr
from oracle import binding as ob
from tests.helpers import camera_sequence
from tests.test_gpu_frames import _compare_frame, _setup

pytestmark = pytest.mark.gpu


def _textured_cornell():
    """The Cornell box with checker textures on every Lambertian material and on
    the light, texture coordinates from the vertex positions."""
    s = xr.Scene.cornell()
    rng = np.random.default_rng(4)
    tex = [rng.integers(0, 256, (5, 7, 4)).astype(np.uint8), rng.integers(64, 256, (16, 3, 4)).astype(np.uint8)]
    v = s.vertices.copy()
    v[:, 6] = v[:, 0] * 0.7 + v[:, 2] * 0.3 + 0.5          # u, partly outside [0, 1]: clamp to edge
    v[:, 7] = v[:, 1] * 0.9 - 0.2
    m = s.materials.copy()
    models = m[:, 7].view(np.uint32)
    for k in range(m.shape[0]):
        if models[k] == 0:
            m[k, 4] = np.array([k % 2], np.int32).view(np.float32)[0]
        elif models[k] == 4:
            m[k, 4] = np.array([1], np.int32).view(np.float32)[0]
    return xr.Scene(v, s.indices, m, s.ranges, s.camera, tex)


@pytest.mark.parametrize("compat", [False, True])
def test_textured_frames_bit_exact(compat):
    scene = _textured_cornell()
    W, H = 96, 72
    pf = xr.params_reference if compat else xr.params_default
    p = pf(W, H, write_hdr=1)

    def move(f, cam):
        cam.position[0] += 0.01
        cam.yaw_deg += 0.2

    r, o = _setup(scene, p)
    with r:
        for f, u in enumerate(camera_sequence(scene, W, H, 3, 4, move=move)):
            r.render(u)
            o.render(u)
            _compare_frame(r, o, compat, f"frame {f}")


def test_textures_change_the_image():
    """Textured materials take the texture, not the base colour."""
    scene = _textured_cornell()
    plain = xr.Scene(scene.vertices, scene.indices, xr.Scene.cornell().materials, scene.ranges, scene.camera)
    W, H = 64, 48
    outs = []
    for s in (scene, plain):
        with xr.Renderer(W, H) as r:
            r.set_params(xr.params_default(W, H, write_hdr=1))
            r.upload_scene(s)
            r.build_bvh()
            r.render(camera_sequence(s, W, H, 1, 4)[0])
            outs.append(r.read_output(xr._lib.XR_OUT_HDR))
    assert not np.array_equal(outs[0], outs[1])


def test_gltf_scene_bit_exact(tmp_path):
    from tests.test_gltf import _fixture
    from xvk_ray_gb300.gltf import load_gltf
    path, _ = _fixture(tmp_path, glb=True)
    scene = load_gltf(path)
    W, H = 64, 48
    p = xr.params_default(W, H, write_hdr=1)
    r, o = _setup(scene, p)
    with r:
        for f, u in enumerate(camera_sequence(scene, W, H, 2, 4)):
            r.render(u)
            o.render(u)
            _compare_frame(r, o, False, f"frame {f}")
