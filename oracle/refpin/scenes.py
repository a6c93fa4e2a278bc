"""The reference's bundled glTF scenes for the tests and the benchmark (TEST
INFRASTRUCTURE).

`convert()` reads a scene from the reference checkout with the package's own
glTF loader (xvk_ray_gb300.gltf.load_gltf) and writes it, in the upload layout,
to oracle/_ref/scenes/<name>.npz (build output kept out of version control, like
the rest of oracle/_ref); `load()` reads that file, converting first where the
checkout is present.  Nothing of the reference is committed: where neither the
checkout nor the converted file exists, load() raises FileNotFoundError and the
tests that want the scene skip.

Every scene gets the reference's default camera: glm::lookAt((0, 1, 3), (0, 1,
0), (0, 1, 0)) for every scene (src/Asset/Scene.cpp:30) -- position (0, 1, 3),
no yaw or pitch -- and the 45-degree field of view of src/main.cpp:45.
"""
from __future__ import annotations

from pathlib import Path

from . import OUT, REFERENCE_ROOT

SCENES = {
    # README.md:7 "Scene1", loaded first by src/main.cpp:56-57 (CC-BY-4.0, see its license.txt)
    "sibenik": "asset/model/sb2/scene.gltf",
    # the bundled Cornell box (src/main.cpp:58-59)
    "cornell_gltf": "asset/model/cb2/scene.gltf",
}
DIR = OUT / "scenes"


def path(name: str) -> Path:
    return DIR / f"{name}.npz"


def convert(name: str) -> Path:
    from xvk_ray_gb300 import _lib as L
    from xvk_ray_gb300.gltf import load_gltf
    src = REFERENCE_ROOT / SCENES[name]
    scene = load_gltf(src)
    cam = L.XrCamera()
    cam.position[:] = [0.0, 1.0, 3.0]
    cam.yaw_deg, cam.pitch_deg, cam.fov_deg = 0.0, 0.0, 45.0
    scene.camera = cam
    DIR.mkdir(parents=True, exist_ok=True)
    dst = path(name)
    scene.save(dst)
    return dst


def convert_all() -> None:
    for name, rel in SCENES.items():
        if (REFERENCE_ROOT / rel).exists():
            convert(name)


def load(name: str):
    from xvk_ray_gb300.api import Scene
    p = path(name)
    if not p.exists():
        if not (REFERENCE_ROOT / SCENES[name]).exists():
            raise FileNotFoundError(f"{name}: neither the reference checkout nor {p} is present")
        convert(name)
    return Scene.load(p)
