"""Build recipe for libxr.so (sm_103a) and the CPU oracle.

Everything is built in-tree: the library into xvk_ray_gb300/_build/, the oracle
into oracle/_build/.  Translation units are compiled in parallel with one
-gencode (compute_103a / sm_103a) and linked with nvcc.  -fmad=false and
-ffp-contract=off keep one rounding per written operation, which the bit-exact
comparisons against the oracle rely on; fused multiply-adds are written out
explicitly where the kernels want them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libxr.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-Xptxas", "-warn-spills",
    f"-I{ROOT / 'include'}", f"-I{CSRC}",
] + os.environ.get("XR_EXTRA_NVCC_FLAGS", "").split()   # e.g. -DXR_TRACE_BLOCK=512 (tuning builds)
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{ROOT / 'include'}", f"-I{CSRC}"]

CU_SOURCES = ["bvh_build.cu", "trace.cu", "trace_noalloc.cu", "restir.cu", "nrc.cu", "cache_api.cu", "batch.cu",
              "instances.cu", "xr_api.cu"]
CXX_SOURCES = ["scene_gen.cpp", "image_io.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libxr.so")


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({' '.join(cmd[:3])} ...):\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "xr.h"]
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
    for src in CXX_SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", *CXX_FLAGS, f"-I{_cuda_include()}", "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    return LIB


def build_oracle(force: bool = False) -> Path:
    # make tracks the dependencies of both libraries (the oracle and its workload generator)
    _run(["make", "-s", "-C", str(ORACLE_DIR)] + (["-B"] if force else []))
    return ORACLE_LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_library(force=force))
    print(build_oracle(force=force))
