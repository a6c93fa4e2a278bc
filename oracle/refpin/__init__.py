"""The reference pin of the oracle: the reference's own ReSTIR GI shader code,
compiled as C++ and run on the CPU (TEST INFRASTRUCTURE).

Recipe.  `build()` reads the shader files below from the reference checkout
(`REFERENCE_ROOT`, overridable with the environment variable XR_REFERENCE_ROOT),
applies a purely mechanical rewrite -- the list in `rewrite()`: nothing of the
shaders' statements, expressions, constants or control flow is changed -- into
oracle/_ref/hlsl/ (build output, kept out of version control), and compiles
oracle/refpin/ref_pin.cpp with them, hlsl_shim.h and hlsl_intrinsics.h into
oracle/_ref/libxr_ref.so, linked to the oracle's library for traversal.  The
reference sources are read where they lie; nothing of them is committed.

What it yields.  Every helper of random.hlsl, ReSTIRGICommon.hlsl, Sampling.hlsl
and BSDF.hlsl, and whole reference-mode frames -- ReSTIRGIInitialSample,
ReSTIRGITemporalReuse and ReSTIRGISpatialReuse with the closest-hit and miss
shaders, bound and sequenced as ApplicationReSTIRGI.cpp / ReSTIRGIPipeline.cpp
do -- computed by the reference's source.  tests/golden/make_ref_fixtures.py
turns runs of it into the committed fixtures tests/golden/ref_*.npz, against
which tests/test_refpin.py checks the oracle (CPU) and tests/test_gpu_refpin.py
the CUDA kernels.  Where /root/reference is absent (the GPU machine) only the
fixtures are used.

What it cannot pin: the hardware's part of the reference -- traversal (RT cores:
the oracle's closest hit, ties to the lowest primitive, is used inside the
harness) and the evaluation order the compiler and driver choose for dot, mul,
normalize, sin/cos, pow, texture filtering and image-format conversion (given
the oracle's conventions in hlsl_intrinsics.h).
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
LIB = OUT / "libxr_ref.so"
REFERENCE_ROOT = Path(os.environ.get("XR_REFERENCE_ROOT", "/root/reference"))

# shader/HLSL/<path>: every file the three ray-generation shaders and the hit
# and miss shaders include
SHADERS = [
    "random.hlsl",
    "ReSTIRGI/ReSTIRGICommon.hlsl",
    "ReSTIRGI/Material.hlsl",
    "ReSTIRGI/Sampling.hlsl",
    "ReSTIRGI/BSDF.hlsl",
    "ReSTIRGI/RayPayload.hlsl",
    "ReSTIRGI/Vertex.hlsl",
    "ReSTIRGI/UBO.hlsl",
    "ReSTIRGI/ReSTIRGIInitialSample.rgen.hlsl",
    "ReSTIRGI/ReSTIRGITemporalReuse.rgen.hlsl",
    "ReSTIRGI/ReSTIRGISpatialReuse.rgen.hlsl",
    "ReSTIRGI/Ray.rchit.hlsl",
    "ReSTIRGI/Ray.rmiss.hlsl",
]

_FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def rewrite(text: str) -> str:
    """The mechanical HLSL -> C++ rewrite, in this order:
    1. drop a UTF-8 byte-order mark and all comments;
    2. drop `#pragma enable_dxr`, `[shader("...")]` attributes, `: register(...)`
       bindings, `: SV_...` semantics, the `[raypayload]` attribute and the
       payload fields' `: read(...)` / `: write(...)` qualifiers;
    3. `cbuffer Name { members };` -> `members` (the block's declarations at
       namespace scope);
    4. parameters `inout T x` / `out T x` -> `T& x`, `in T x` -> `T x`;
    5. swizzles `.xyz`, `.xy`, `.rgb` -> `.xyz()`, `.xy()`, `.rgb()`;
    6. unsized resource arrays `T name[]` -> `T name[hlsl::kMaxTextures]`;
    7. unsuffixed floating literals `1.0` -> `HLSL_LIT(1.0)` (HLSL literal-float
       typing, see hlsl_shim.h);
    8. vector constructors `float2(a, b)` -> `float2{a, b}`: HLSL evaluates a
       constructor's operands left to right (`float2(RandomFloat(s),
       RandomFloat(s))` takes the first draw for x), which C++ guarantees only
       for brace initialisation."""
    if text.startswith("\xef\xbb\xbf"):
        text = text[3:]
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"^\s*#pragma\s+enable_dxr\s*$", "", text, flags=re.M)
    text = re.sub(r"\[shader\(\"[^\"]*\"\)\]", "", text)
    text = re.sub(r"\s*:\s*register\s*\([^)]*\)", "", text)
    text = re.sub(r"\s*:\s*SV_\w+", "", text)
    text = re.sub(r"struct\s+\[raypayload\]\s+", "struct ", text)
    text = re.sub(r"\s*:\s*(?:read|write)\s*\([^)]*\)", "", text)
    text = re.sub(r"cbuffer\s+\w+\s*\{(.*?)\}\s*;", r"\1", text, flags=re.S)
    text = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)", r"\1& \2", text)
    text = re.sub(r"\bin\s+(\w+)\s+(\w+)", r"\1 \2", text)
    text = re.sub(r"\.(xyz|xy|rgb)\b(?!\s*\()", r".\1()", text)
    text = re.sub(r"(\b\w+\s+\w+)\[\]\s*;", r"\1[hlsl::kMaxTextures];", text)
    text = _FLOAT_LIT.sub(r"HLSL_LIT(\1)", text)
    return _brace_constructors(text)


_VEC_CTOR = re.compile(r"\b((?:float|int|uint)[234])\s*\(")


def _brace_constructors(text: str) -> str:
    out, i = [], 0
    while True:
        m = _VEC_CTOR.search(text, i)
        if not m:
            out.append(text[i:])
            return "".join(out)
        # the matching parenthesis (declarations such as `float3 Mix(` never match: a name sits between)
        j, depth = m.end(), 1
        while depth:
            c = text[j]
            depth += c == "("
            depth -= c == ")"
            j += 1
        out.append(text[i:m.start()])
        out.append(m.group(1) + "{" + _brace_constructors(text[m.end():j - 1]) + "}")
        i = j


def available() -> bool:
    return (REFERENCE_ROOT / "shader" / "HLSL" / "ReSTIRGI" / "ReSTIRGICommon.hlsl").exists()


def build(force: bool = False) -> Path:
    """Rewrites the reference's shaders into oracle/_ref/hlsl and builds
    oracle/_ref/libxr_ref.so (needs the reference checkout and the oracle's
    library, oracle/_build/liboracle.so)."""
    src = REFERENCE_ROOT / "shader" / "HLSL"
    if not available():
        raise FileNotFoundError(f"reference shaders not found under {src}")
    subprocess.run(["make", "-s", "-C", str(ORACLE)], check=True)
    hl = OUT / "hlsl"
    changed = force or not LIB.exists()
    for rel in SHADERS:
        text = (src / rel).read_bytes().decode("latin-1")
        out = rewrite(text).encode("latin-1")
        dst = hl / rel
        if not dst.exists() or dst.read_bytes() != out:
            dst.parent.mkdir(parents=True, exist_ok=True)
            dst.write_bytes(out)
            changed = True
    deps = [HERE / "ref_pin.cpp", HERE / "hlsl_shim.h", HERE / "hlsl_intrinsics.h", ORACLE / "xr_oracle.h",
            ORACLE / "_build" / "liboracle.so"]
    if not changed and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    # -ftrivial-auto-var-init=zero: what the shaders leave undefined (InitSample
    # sets neither p_q, f nor the pad words of a sample; an OpUndef in SPIR-V)
    # reads as zero, as in the oracle
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-ftrivial-auto-var-init=zero", "-w", f"-I{HERE}", f"-I{ORACLE}", f"-I{hl}", str(HERE / "ref_pin.cpp"),
           f"-L{ORACLE / '_build'}", "-loracle", "-Wl,-rpath,$ORIGIN/../_build", "-o", str(LIB)]
    subprocess.run(cmd, check=True)
    return LIB


# ---------------------------------------------------------------------------
# ctypes binding
# ---------------------------------------------------------------------------
_lib = None


def load():
    global _lib
    if _lib is None:
        from oracle import binding as ob
        ob.load()   # liboracle.so first (the pin resolves or_trace from it)
        lib = C.CDLL(str(LIB))
        P, u32, f32 = C.c_void_p, C.c_uint32, C.c_float
        sig = {
            "ref_scene_create": (P, [P, u32, P, u32, P, u32, P, u32]),
            "ref_scene_set_textures": (None, [P, P, u32, P]),
            "ref_scene_destroy": (None, [P]),
            "ref_renderer_create": (P, [P, u32, u32]),
            "ref_renderer_destroy": (None, [P]),
            "ref_render_frame": (None, [P, P]),
            "ref_run_pass": (None, [P, P, C.c_int, P, P]),
            "ref_set_gbuffer_from_samples": (None, [P, P, P]),
            "ref_read": (C.c_size_t, [P, C.c_int, P, C.c_size_t]),
            "ref_write": (C.c_int, [P, C.c_int, P, C.c_size_t]),
            "ref_init_random_seed": (u32, [u32, u32, u32, u32, u32]),
            "ref_random_sequence": (None, [u32, u32, P, P, P, P]),
            "ref_onb": (None, [P, u32, P]),
            "ref_sample_hemisphere": (None, [P, u32, P]),
            "ref_sample_bsdf": (None, [P, P, P, P, u32, P]),
            "ref_evaluate_bsdf": (None, [P, P, P, P, u32, P]),
            "ref_update_list": (None, [P, P, u32, u32, P, P, P]),
            "ref_merge_list": (None, [P, P, u32, u32, P, P, P]),
            "ref_similar": (None, [P, P, u32, P]),
            "ref_aces": (None, [P, u32, P]),
            "ref_target_pdf": (None, [P, P, P, P, u32, P]),
            "ref_eval_target": (None, [P, P, P, u32, P]),
            "ref_world_to_screen_uv": (None, [P, u32, P, P, P]),
            "ref_neighbor_index": (None, [u32, u32, u32, u32, f32, u32, u32, P]),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype, f.argtypes = r, a
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data if a is not None and a.size else None


BUF_SAMPLES, BUF_TEMPORAL, BUF_SPATIAL, BUF_OUTPUT, BUF_GPOS, BUF_MOTION, BUF_GNRM, BUF_GMATUV = range(8)


class RefScene:
    """A scene in the reference's buffers: AVertex words, per-model local
    indices and {indexOffset, vertexOffset} offsets, AMaterial words."""

    def __init__(self, scene):
        lib = load()
        v = np.ascontiguousarray(scene.vertices, np.float32).view(np.uint32)
        i = np.ascontiguousarray(scene.indices, np.uint32)
        m = np.ascontiguousarray(scene.materials, np.float32).view(np.uint32)
        rg = np.ascontiguousarray(scene.ranges, np.uint32).reshape(-1, 2)
        self._keep = (v, i, m, rg)
        self.ptr = lib.ref_scene_create(_p(v), v.shape[0], _p(i), i.size, _p(m), m.shape[0], _p(rg), rg.shape[0])
        tex = getattr(scene, "textures", None)
        if tex:
            sizes = np.array([[t.shape[1], t.shape[0]] for t in tex], np.uint32)
            texels = np.ascontiguousarray(np.concatenate([np.ascontiguousarray(t, np.uint8).reshape(-1) for t in tex]))
            lib.ref_scene_set_textures(self.ptr, _p(sizes), len(tex), _p(texels))

    def close(self):
        if self.ptr:
            load().ref_scene_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RefRenderer:
    """ApplicationReSTIRGI's three passes on the CPU, with the reference's own shader code."""

    def __init__(self, scene: RefScene, width: int, height: int):
        self.scene = scene
        self.W, self.H = width, height
        self.ptr = load().ref_renderer_create(scene.ptr, width, height)

    def render(self, ubo) -> None:
        load().ref_render_frame(self.ptr, C.addressof(ubo))

    def run_pass(self, ubo, pass_id: int, samples: np.ndarray | None = None,
                 temporal: np.ndarray | None = None) -> None:
        s = None if samples is None else np.ascontiguousarray(samples, np.uint32)
        t = None if temporal is None else np.ascontiguousarray(temporal, np.uint32)
        load().ref_run_pass(self.ptr, C.addressof(ubo), pass_id, _p(s), _p(t))

    def set_gbuffer_from_samples(self, ubo, samples: np.ndarray) -> None:
        s = np.ascontiguousarray(samples, np.uint32)
        load().ref_set_gbuffer_from_samples(self.ptr, C.addressof(ubo), _p(s))

    def write(self, which: int, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr)
        if load().ref_write(self.ptr, which, _p(a), a.nbytes) != 0:
            raise ValueError("ref_write: bad buffer or size")

    def read(self, which: int) -> np.ndarray:
        lib = load()
        n = lib.ref_read(self.ptr, which, None, 0)
        if which in (BUF_SAMPLES, BUF_TEMPORAL, BUF_SPATIAL):
            out = np.empty(n // 4, np.uint32)
            lib.ref_read(self.ptr, which, _p(out), n)
            return out.reshape(-1, 24 if which == BUF_SAMPLES else 28)
        out = np.empty(n // 4, np.float32)
        lib.ref_read(self.ptr, which, _p(out), n)
        return out.reshape(-1, 2 if which == BUF_MOTION else 4)

    def close(self):
        if self.ptr:
            load().ref_renderer_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
