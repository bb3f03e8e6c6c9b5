"""In-tree build of the native libraries.

* ``libopenph_gb300.so`` — the CUDA reduction library and its C ABI
  (``include/openph.h``), compiled by nvcc for sm_103a only.
* ``libophgen.so`` — host-only complex generators (``gen/ophgen.c``).

Everything is compiled into the package directory; nothing is installed.
The translation units are compiled in parallel and linked once.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
GEN = PKG / "gen"
BUILD = PKG / "_build"
LIB = PKG / "libopenph_gb300.so"
GENLIB = PKG / "libophgen.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(CSRC)]

CU_SOURCES = sorted(CSRC.glob("*.cu"))
HEADERS = sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build openph_gb300")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def build_gen(force: bool = False) -> Path:
    src = GEN / "ophgen.c"
    if force or _stale(GENLIB, [src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fvisibility=hidden",
              "-Wall", "-pthread", "-o", str(GENLIB), str(src), "-lm"])
    return GENLIB


def build_cuda(force: bool = False, extra_flags=()) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    objs = []
    jobs = []
    for src in CU_SOURCES:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *HEADERS]):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
    return LIB


def build_all(force: bool = False) -> None:
    build_gen(force)
    build_cuda(force)
