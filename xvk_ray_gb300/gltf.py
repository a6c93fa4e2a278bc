"""glTF 2.0 scenes (.gltf + buffers, .glb) and PNG base-colour textures.

Follows the reference's loader (src/Asset/Model.cpp:97-234, AglTFModel):

* the first scene's node hierarchy; a node's matrix is `matrix` when given, else
  T(translation) * R(rotation quaternion) * S(scale), composed with its parents'
  (parent * child);
* per primitive: POSITION transformed by the node matrix, NORMAL by its inverse
  transpose (of the normalised normal, w = 1, not re-normalised: the hit shader
  normalises), TEXCOORD_0 (else 0), indices of 8, 16 or 32 bits offset by the
  primitive's first vertex, the primitive's material index on every vertex;
* materials: pbrMetallicRoughness.baseColorFactor (default 1), baseColorTexture's
  texture index (else -1), model DiffuseLight for a material named "light", else
  Lambertian (src/Asset/Model.cpp:66-95);
* textures -> images decoded to RGBA8 (src/Asset/Model.cpp:19-58), row 0 of the
  image at texture coordinate v = 0.

Where the reference's loader would mis-read a valid file this one does the
specified thing instead: accessor byteStride is honoured (the reference assumes
tightly packed attributes), RGB images are expanded to RGBA (the reference drops
their texels), a primitive without material gets a default white Lambertian
material, and a primitive without normals gets area-weighted vertex normals
(the reference would normalise a zero vector).  Images must be PNG (JPEG needs a
decoder this build does not carry: convert the textures to PNG).
"""
from __future__ import annotations

import base64
import json
import struct
import zlib
from pathlib import Path

import numpy as np

from . import _lib as L
from .api import Scene, _ptr

_COMPONENTS = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}
_DTYPES = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}


# ---------------------------------------------------------------------------
# PNG
# ---------------------------------------------------------------------------
def decode_png(data: bytes) -> np.ndarray:
    """PNG (bit depth 1..16, colour types 0/2/3/4/6, not interlaced) -> (h, w, 4) uint8 RGBA."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, plte, trns = 8, bytearray(), None, None
    w = h = depth = ctype = interlace = 0
    while pos + 8 <= len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body[:13])
        elif tag == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif tag == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif tag == b"IDAT":
            idat += body
        elif tag == b"IEND":
            break
        pos += 12 + n
    if interlace:
        raise ValueError("interlaced PNG is not supported")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bits = channels * depth
    row_bytes = (w * bits + 7) // 8
    bpp = max(1, bits // 8)
    raw = zlib.decompress(bytes(idat))
    if len(raw) < h * (row_bytes + 1):
        raise ValueError("truncated PNG image data")
    src = np.frombuffer(raw, np.uint8)
    rows = np.empty(h * row_bytes, np.uint8)
    st = L.load().xr_png_unfilter(_ptr(src), h, row_bytes, bpp, _ptr(rows))
    if st != L.XR_OK:
        raise ValueError("bad PNG filter type")
    rows = rows.reshape(h, row_bytes)
    if depth == 16:
        samples = rows.reshape(h, w * channels, 2)[:, :, 0]          # high byte
    elif depth == 8:
        samples = rows.reshape(h, w * channels)
    else:                                                           # 1, 2, 4 bits: gray or palette
        per = 8 // depth
        bitsarr = np.unpackbits(rows, axis=1)
        vals = bitsarr.reshape(h, -1, depth)
        weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint8)
        samples = (vals * weights).sum(axis=2).astype(np.uint8)[:, :w * channels]
        if ctype == 0:
            samples = (samples.astype(np.uint32) * 255 // ((1 << depth) - 1)).astype(np.uint8)
        del per
    px = samples.reshape(h, w, channels)
    out = np.empty((h, w, 4), np.uint8)
    if ctype == 3:
        if plte is None:
            raise ValueError("palette PNG without PLTE")
        idx = px[:, :, 0]
        out[:, :, :3] = plte[idx]
        alpha = np.full(256, 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = trns
        out[:, :, 3] = alpha[idx]
    elif ctype == 0:
        out[:, :, :3] = px[:, :, :1]
        out[:, :, 3] = 255
    elif ctype == 4:
        out[:, :, :3] = px[:, :, :1]
        out[:, :, 3] = px[:, :, 1]
    elif ctype == 2:
        out[:, :, :3] = px
        out[:, :, 3] = 255
    else:
        out[:] = px
    return out


# ---------------------------------------------------------------------------
# glTF
# ---------------------------------------------------------------------------
def _mat_trs(node) -> np.ndarray:
    if "matrix" in node:
        return np.array(node["matrix"], np.float64).reshape(4, 4).T      # column-major
    m = np.eye(4)
    if "translation" in node:
        t = np.eye(4)
        t[:3, 3] = node["translation"]
        m = m @ t
    if "rotation" in node:
        x, y, z, w = node["rotation"]
        r = np.eye(4)
        r[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
        m = m @ r
    if "scale" in node:
        m = m @ np.diag(list(node["scale"]) + [1.0])
    return m


class _Doc:
    def __init__(self, path: Path):
        self.path = Path(path)
        data = self.path.read_bytes()
        self.bin = None
        if data[:4] == b"glTF":
            _, _, length = struct.unpack("<4sII", data[:12])
            pos = 12
            while pos < length:
                clen, ctype = struct.unpack("<I4s", data[pos:pos + 8])
                chunk = data[pos + 8:pos + 8 + clen]
                if ctype == b"JSON":
                    self.j = json.loads(chunk.decode("utf-8"))
                elif ctype == b"BIN\x00":
                    self.bin = chunk
                pos += 8 + clen
        else:
            self.j = json.loads(data.decode("utf-8"))
        self.buffers = []
        for b in self.j.get("buffers", []):
            uri = b.get("uri")
            if uri is None:
                self.buffers.append(self.bin)
            elif uri.startswith("data:"):
                self.buffers.append(base64.b64decode(uri.split(",", 1)[1]))
            else:
                self.buffers.append((self.path.parent / uri).read_bytes())

    def view_bytes(self, vi: int) -> tuple[bytes, int]:
        v = self.j["bufferViews"][vi]
        buf = self.buffers[v["buffer"]]
        off = v.get("byteOffset", 0)
        return buf[off:off + v["byteLength"]], v.get("byteStride", 0)

    def accessor(self, ai: int) -> np.ndarray:
        a = self.j["accessors"][ai]
        if "sparse" in a:
            raise ValueError("sparse accessors are not supported")
        dt = np.dtype(_DTYPES[a["componentType"]])
        nc = _COMPONENTS[a["type"]]
        count = a["count"]
        if "bufferView" not in a:
            return np.zeros((count, nc), dt)
        data, stride = self.view_bytes(a["bufferView"])
        off = a.get("byteOffset", 0)
        elem = dt.itemsize * nc
        stride = stride or elem
        raw = np.frombuffer(data, np.uint8, count=(count - 1) * stride + elem, offset=off) if count else np.zeros(0, np.uint8)
        if stride == elem:
            return raw.view(dt).reshape(count, nc).copy()
        rows = np.lib.stride_tricks.as_strided(raw, shape=(count, elem), strides=(stride, 1))
        return np.ascontiguousarray(rows).view(dt).reshape(count, nc)

    def image(self, ii: int) -> np.ndarray:
        im = self.j["images"][ii]
        if "uri" in im:
            uri = im["uri"]
            data = base64.b64decode(uri.split(",", 1)[1]) if uri.startswith("data:") else (self.path.parent / uri).read_bytes()
        else:
            data, _ = self.view_bytes(im["bufferView"])
        if data[:8] != b"\x89PNG\r\n\x1a\n":
            raise ValueError(f"image {ii}: only PNG images are supported (convert JPEG textures to PNG)")
        return decode_png(data)


def _vertex_normals(pos: np.ndarray, idx: np.ndarray) -> np.ndarray:
    tri = idx.reshape(-1, 3)
    fn = np.cross(pos[tri[:, 1]] - pos[tri[:, 0]], pos[tri[:, 2]] - pos[tri[:, 0]])
    n = np.zeros_like(pos)
    for k in range(3):
        np.add.at(n, tri[:, k], fn)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    return np.where(ln > 0, n / np.where(ln > 0, ln, 1), np.array([0.0, 1.0, 0.0]))


def load_gltf(path, camera: L.XrCamera | None = None) -> Scene:
    """A glTF 2.0 file as a Scene (vertices, global indices, materials, RGBA8 textures)."""
    d = _Doc(path)
    j = d.j
    verts, idxs = [], []
    n_vert = 0
    mats_json = j.get("materials", [])
    default_mat = len(mats_json)          # appended if a primitive has no material
    need_default = False

    def visit(ni: int, parent: np.ndarray):
        nonlocal n_vert, need_default
        node = j["nodes"][ni]
        m = parent @ _mat_trs(node)
        if "mesh" in node:
            nmat = np.linalg.inv(m).T
            for prim in j["meshes"][node["mesh"]]["primitives"]:
                if prim.get("mode", 4) != 4:
                    continue                                       # triangles only
                attr = prim["attributes"]
                p = d.accessor(attr["POSITION"]).astype(np.float64)
                if "indices" in prim:
                    ix = d.accessor(prim["indices"]).reshape(-1).astype(np.uint64)
                else:
                    ix = np.arange(len(p), dtype=np.uint64)
                if "NORMAL" in attr:
                    nrm = d.accessor(attr["NORMAL"]).astype(np.float64)
                    ln = np.linalg.norm(nrm, axis=1, keepdims=True)
                    nrm = nrm / np.where(ln > 0, ln, 1.0)
                else:
                    nrm = _vertex_normals(p, ix.astype(np.int64))
                uv = d.accessor(attr["TEXCOORD_0"]).astype(np.float64) if "TEXCOORD_0" in attr else np.zeros((len(p), 2))
                mi = prim.get("material")
                if mi is None:
                    mi = default_mat
                    need_default = True
                ph = np.concatenate([p, np.ones((len(p), 1))], 1) @ m.T
                nh = np.concatenate([nrm, np.ones((len(p), 1))], 1) @ nmat.T
                v = np.zeros((len(p), 9), np.float32)
                v[:, 0:3] = ph[:, :3]
                v[:, 3:6] = nh[:, :3]
                v[:, 6:8] = uv
                v[:, 8] = np.array([mi], np.int32).view(np.float32)[0]
                verts.append(v)
                idxs.append((ix + n_vert).astype(np.uint32))
                n_vert += len(p)
        for c in node.get("children", []):
            visit(c, m)

    scene_i = j.get("scene", 0)
    roots = j["scenes"][scene_i]["nodes"] if j.get("scenes") else range(len(j.get("nodes", [])))
    for ni in roots:
        visit(ni, np.eye(4))
    textures_json = j.get("textures", [])
    mats = np.zeros((len(mats_json) + (1 if need_default else 0), 8), np.float32)
    for k, mj in enumerate(mats_json):
        pbr = mj.get("pbrMetallicRoughness", {})
        mats[k, 0:4] = pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0])
        tex = pbr.get("baseColorTexture", {}).get("index", -1)
        mats[k, 4] = np.array([tex], np.int32).view(np.float32)[0]
        model = L.XR_MAT_DIFFUSE_LIGHT if mj.get("name") == "light" else L.XR_MAT_LAMBERTIAN
        mats[k, 7] = np.array([model], np.uint32).view(np.float32)[0]
    if need_default:
        mats[-1, 0:4] = 1.0
        mats[-1, 4] = np.array([-1], np.int32).view(np.float32)[0]
    textures = [d.image(t["source"]) for t in textures_json]
    vertices = np.concatenate(verts) if verts else np.zeros((0, 9), np.float32)
    indices = np.concatenate(idxs) if idxs else np.zeros(0, np.uint32)
    if camera is None:
        camera = L.XrCamera.from_buffer_copy(Scene.cornell().camera)
    return Scene(vertices, indices, mats, np.zeros((1, 2), np.uint32), camera, textures)
