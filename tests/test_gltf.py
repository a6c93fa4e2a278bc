"""glTF 2.0 / PNG scene loading (xvk_ray_gb300.gltf) on the CPU.

Files are generated here (own content); the reference's bundled Cornell box is
parsed when its asset directory is present.
"""
import base64
import json
import math
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

import xvk_ray_gb300 as xr
from xvk_ray_gb300 import _lib as L
from xvk_ray_gb300.gltf import decode_png, load_gltf


# ---- a PNG encoder with every filter type (the decoder's checker) ----
def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _encode_png(samples: np.ndarray, ctype: int, depth: int, rng, plte=None, trns=None) -> bytes:
    """samples: (h, row_bytes) uint8 of already packed rows."""
    h, rb = samples.shape
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp = max(1, channels * depth // 8)
    out = bytearray()
    prev = np.zeros(rb, np.int32)
    for y in range(h):
        row = samples[y].astype(np.int32)
        ft = int(rng.integers(0, 5))
        f = np.zeros(rb, np.int32)
        for i in range(rb):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            f[i] = (row[i] - pred) & 255
        out += bytes([ft]) + bytes(f.astype(np.uint8))
        prev = row
    w = rb * 8 // (channels * depth)

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if plte is not None:
        png += chunk(b"PLTE", bytes(plte.astype(np.uint8).reshape(-1)))
    if trns is not None:
        png += chunk(b"tRNS", bytes(trns.astype(np.uint8)))
    return png + chunk(b"IDAT", zlib.compress(bytes(out))) + chunk(b"IEND", b"")


@pytest.mark.parametrize("ctype", [0, 2, 3, 4, 6])
def test_png_decode_filters_and_colour_types(ctype):
    rng = np.random.default_rng(ctype)
    h, w = 7, 9
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    px = rng.integers(0, 256 if ctype != 3 else 5, (h, w, ch)).astype(np.uint8)
    plte = trns = None
    if ctype == 3:
        plte = rng.integers(0, 256, (5, 3))
        trns = np.array([0, 128, 255])
    data = _encode_png(px.reshape(h, w * ch), ctype, 8, rng, plte, trns)
    got = decode_png(data)
    assert got.shape == (h, w, 4)
    if ctype == 0:
        exp = np.concatenate([px.repeat(3, 2), np.full((h, w, 1), 255, np.uint8)], 2)
    elif ctype == 2:
        exp = np.concatenate([px, np.full((h, w, 1), 255, np.uint8)], 2)
    elif ctype == 4:
        exp = np.concatenate([px[:, :, :1].repeat(3, 2), px[:, :, 1:]], 2)
    elif ctype == 6:
        exp = px
    else:
        alpha = np.array([0, 128, 255, 255, 255], np.uint8)
        exp = np.concatenate([plte.astype(np.uint8)[px[:, :, 0]], alpha[px[:, :, 0]][:, :, None]], 2)
    assert np.array_equal(got, exp)


def test_png_decode_16_bit_and_1_bit():
    rng = np.random.default_rng(5)
    h, w = 4, 6
    px16 = rng.integers(0, 65536, (h, w * 3)).astype(">u2")
    got = decode_png(_encode_png(px16.view(np.uint8).reshape(h, -1), 2, 16, rng))
    assert np.array_equal(got[:, :, :3], (px16.astype(np.uint32) >> 8).astype(np.uint8).reshape(h, w, 3))
    bits = rng.integers(0, 2, (h, 16)).astype(np.uint8)
    got1 = decode_png(_encode_png(np.packbits(bits, axis=1), 0, 1, rng))
    assert np.array_equal(got1[:, :, 0], bits * 255)


# ---- glTF fixture ----
def _fixture(tmp_path: Path, glb: bool):
    """A textured quad under a translated + rotated + scaled parent node, a light
    triangle, interleaved position/normal/uv (byteStride 32), uint16 indices."""
    quad_p = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], np.float32)
    quad_n = np.tile(np.array([[0, 1, 0]], np.float32), (4, 1))
    quad_uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    inter = np.concatenate([quad_p, quad_n, quad_uv], 1).astype(np.float32)        # 8 floats = 32 B
    qidx = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    lp = np.array([[0, 2, 0], [0.5, 2, 0], [0, 2, 0.5]], np.float32)
    lidx = np.array([0, 1, 2], np.uint32)
    blob = inter.tobytes() + qidx.tobytes() + b"\x00\x00" + lp.tobytes() + lidx.tobytes()
    off_q = 0
    off_qi = inter.nbytes
    off_lp = off_qi + qidx.nbytes + 2
    off_li = off_lp + lp.nbytes
    tex = np.zeros((2, 2, 4), np.uint8)
    tex[0, 0] = [255, 0, 0, 255]; tex[0, 1] = [0, 255, 0, 255]; tex[1, 0] = [0, 0, 255, 255]; tex[1, 1] = [255, 255, 255, 255]
    from xvk_ray_gb300.render import write_png
    write_png(str(tmp_path / "checker.png"), tex.reshape(-1, 4), 2, 2)
    j = {
        "asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0, 2]}],
        "nodes": [{"translation": [0, 1, 0], "rotation": [0, math.sin(math.pi / 4), 0, math.cos(math.pi / 4)],
                   "scale": [2, 2, 2], "children": [1]},
                  {"mesh": 0}, {"mesh": 1}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2}, "indices": 3,
                                    "material": 0}]},
                   {"primitives": [{"attributes": {"POSITION": 4}, "indices": 5, "material": 1}]}],
        "materials": [{"name": "floor", "pbrMetallicRoughness": {"baseColorFactor": [0.5, 0.5, 0.5, 1],
                                                                 "baseColorTexture": {"index": 0}}},
                      {"name": "light", "pbrMetallicRoughness": {"baseColorFactor": [4, 3, 2, 1]}}],
        "textures": [{"source": 0}], "images": [{"uri": "checker.png"}],
        "buffers": [{"byteLength": len(blob)}],
        "bufferViews": [{"buffer": 0, "byteOffset": off_q, "byteLength": inter.nbytes, "byteStride": 32},
                        {"buffer": 0, "byteOffset": off_qi, "byteLength": qidx.nbytes},
                        {"buffer": 0, "byteOffset": off_lp, "byteLength": lp.nbytes},
                        {"buffer": 0, "byteOffset": off_li, "byteLength": lidx.nbytes}],
        "accessors": [{"bufferView": 0, "byteOffset": 0, "componentType": 5126, "count": 4, "type": "VEC3"},
                      {"bufferView": 0, "byteOffset": 12, "componentType": 5126, "count": 4, "type": "VEC3"},
                      {"bufferView": 0, "byteOffset": 24, "componentType": 5126, "count": 4, "type": "VEC2"},
                      {"bufferView": 1, "componentType": 5123, "count": 6, "type": "SCALAR"},
                      {"bufferView": 2, "componentType": 5126, "count": 3, "type": "VEC3"},
                      {"bufferView": 3, "componentType": 5125, "count": 3, "type": "SCALAR"}],
    }
    if glb:
        jb = json.dumps(j).encode()
        jb += b" " * (-len(jb) % 4)
        bb = blob + b"\x00" * (-len(blob) % 4)
        data = struct.pack("<4sII", b"glTF", 2, 12 + 8 + len(jb) + 8 + len(bb))
        data += struct.pack("<I4s", len(jb), b"JSON") + jb + struct.pack("<I4s", len(bb), b"BIN\x00") + bb
        path = tmp_path / "scene.glb"
        path.write_bytes(data)
    else:
        j["buffers"][0]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(blob).decode()
        path = tmp_path / "scene.gltf"
        path.write_text(json.dumps(j))
    return path, tex


@pytest.mark.parametrize("glb", [False, True])
def test_gltf_fixture(tmp_path, glb):
    path, tex = _fixture(tmp_path, glb)
    s = load_gltf(path)
    assert s.n_triangles == 3
    v = s.vertices
    # quad: scale 2, rotate 90 deg about y, translate (0, 1, 0)
    m_rot = np.array([[0, 0, 1], [0, 1, 0], [-1, 0, 0]], np.float64)
    p0 = m_rot @ (2.0 * np.array([-1.0, 0.0, -1.0])) + np.array([0, 1, 0])
    assert np.allclose(v[0, 0:3], p0, atol=1e-6)
    # normal by the inverse transpose (not re-normalised): (0, 1, 0) / 2
    assert np.allclose(v[0, 3:6], [0, 0.5, 0], atol=1e-6)
    assert np.array_equal(v[:4, 6:8], [[0, 0], [1, 0], [1, 1], [0, 1]])
    assert np.array_equal(v[:4, 8].view(np.int32), [0] * 4) and np.array_equal(v[4:, 8].view(np.int32), [1] * 3)
    # the light primitive has no normals: area-weighted vertex normals of its triangle
    assert np.allclose(np.abs(v[4, 3:6]), [0, 1, 0], atol=1e-6)
    assert np.array_equal(s.indices, [0, 1, 2, 0, 2, 3, 4, 5, 6])
    m = s.materials
    assert m[0, 4].view(np.int32) == 0 and m[0, 7].view(np.uint32) == L.XR_MAT_LAMBERTIAN
    assert m[1, 7].view(np.uint32) == L.XR_MAT_DIFFUSE_LIGHT and m[1, 4].view(np.int32) == -1
    assert np.allclose(m[1, 0:4], [4, 3, 2, 1])
    assert len(s.textures) == 1 and np.array_equal(s.textures[0], tex)


def test_gltf_reference_cornell_box():
    """The reference's bundled Cornell box (asset/model/cb2) when the asset is present."""
    from oracle.refpin import REFERENCE_ROOT
    p = REFERENCE_ROOT / "asset" / "model" / "cb2" / "scene.gltf"
    if not p.exists():
        pytest.skip("reference assets not present")
    s = load_gltf(p)
    assert s.n_triangles == 32
    models = s.materials[:, 7].view(np.uint32)
    assert (models == L.XR_MAT_DIFFUSE_LIGHT).sum() == 1
    assert np.all(np.isfinite(s.vertices))
