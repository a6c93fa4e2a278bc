"""Headless renderer: frames of a scene through the C ABI, PNG output.

The reference presents its output image to a swap chain
(src/Vulkan/RayTracing/ApplicationReSTIRGI.cpp:248-271) and vendors
stb_image_write.h without using it; here the tone-mapped RGBA8 image of the
last frame is written as a PNG file (8-bit RGBA, zlib-compressed scanlines with
filter type 0).

    python -m xvk_ray_gb300.render --scene procedural --frames 12 --cache --png out.png
"""
from __future__ import annotations

import argparse
import struct
import sys
import time
import zlib

import numpy as np

from . import _lib as L
from .api import Renderer, Scene, cache_params_default, camera_ubo, params_default

# the benchmark scene: ground plane, 4096 icospheres/boxes, 16 emissive quads
PROCEDURAL_1M = dict(seed=1, n_objects=4096, n_lights=16, extent=40.0, sphere_subdiv=2)


def write_png(path: str, rgba: np.ndarray, width: int, height: int) -> None:
    """RGBA8 pixels (row 0 = top row of the file) as a PNG file."""
    img = np.ascontiguousarray(rgba, np.uint8).reshape(height, width, 4)
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(height))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    hdr = struct.pack(">IIBBBBB", width, height, 8, 6, 0, 0, 0)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", hdr) + chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def read_png_rgba(path: str) -> tuple[np.ndarray, int, int]:
    """Reads back what write_png writes (8-bit RGBA, filter type 0)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG file"
    pos, idat = 8, b""
    w = h = 0
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 6, "only 8-bit RGBA"
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    assert np.all(raw[:, 0] == 0), "only filter type 0"
    return raw[:, 1:].reshape(h * w, 4).copy(), w, h


def camera_path(scene: Scene, width: int, height: int, frames: int, bounces: int, move: bool):
    """UBOs of the benchmark camera path (0.01 units and 0.2 degrees of yaw per frame)."""
    cam = L.XrCamera.from_buffer_copy(scene.camera)
    prev, out = None, []
    for f in range(frames):
        if move:
            cam.position[2] -= 0.01
            cam.yaw_deg += 0.2
        u = camera_ubo(cam, width, height, prev, f, bounces, sky=False, reuse=True)
        prev = u
        out.append(u)
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--scene", choices=["procedural", "cornell"], default="procedural")
    ap.add_argument("--gltf", default=None, help="render this glTF 2.0 file (.gltf / .glb) instead")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--frames", type=int, default=12)
    ap.add_argument("--bounces", type=int, default=4)
    ap.add_argument("--static", action="store_true", help="keep the camera still")
    ap.add_argument("--cache", action="store_true", help="enable the learned radiance cache")
    ap.add_argument("--png", default=None, help="write the last frame's tone-mapped image here")
    a = ap.parse_args(argv)
    if a.gltf:
        from .gltf import load_gltf
        scene = load_gltf(a.gltf)
    else:
        scene = Scene.procedural(**PROCEDURAL_1M) if a.scene == "procedural" else Scene.cornell()
    ubos = camera_path(scene, a.width, a.height, a.frames, a.bounces, not a.static)
    with Renderer(a.width, a.height) as r:
        r.set_params(params_default(a.width, a.height))
        r.upload_scene(scene)
        r.build_bvh()
        if a.cache:
            cp = cache_params_default()
            cp.enabled = 1
            r.cache.set_params(cp)
        t0 = time.perf_counter()
        for u in ubos:
            r.render(u)
        img = r.read_output(L.XR_OUT_LDR8)
        wall = time.perf_counter() - t0
        st = r.stats()
        print(f"{a.frames} frames {a.width}x{a.height}: last frame {st.ms_frame:.3f} ms on the device, "
              f"{1e3 * wall / a.frames:.3f} ms per frame wall", flush=True)
        if a.cache:
            cs = r.cache.stats()
            print(f"cache: {cs.steps} Adam steps, loss {cs.loss:.4f}, {cs.queries} queries, "
                  f"{cs.train_samples} training samples", flush=True)
    if a.png:
        write_png(a.png, img, a.width, a.height)
        print(f"wrote {a.png}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
