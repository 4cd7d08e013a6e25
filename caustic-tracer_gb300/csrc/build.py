"""Builds libcaustic_gb300.so for sm_103a into caustic-tracer_gb300/_build/.

Each translation unit is compiled by its own nvcc process (in parallel), then
linked into one shared library. Host C++ is compiled with -ffp-contract=off so
the packer's float64 arithmetic rounds exactly like the reference's. Device
code is compiled with -fmad=false: the compiler fuses no multiply-add on its
own (its choice could differ between kernels that inline the same function),
and hot code writes the fused forms it wants with __fmaf_rn.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
PKG = HERE.parent
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libcaustic_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
SOURCES = ["pack_host.cpp", "profile.cpp", "scene.cu", "trace.cu", "integrator.cu", "batch.cu", "display.cu"]
HEADERS = ["common.hpp", "scene.hpp", "traverse.cuh", "integrator.cuh", "wavefront.cuh", "profile.hpp",
           "../../include/caustic.h"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not pathlib.Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libcaustic_gb300")
    return cand


def _compile(src: str, obj: pathlib.Path) -> None:
    path = HERE / src
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
              f"-I{HERE}", f"-I{PKG.parent / 'include'}"]
    if src.endswith(".cu"):
        cmd = [nvcc(), ARCH, "-lineinfo", "-fmad=false", "-Xptxas", "-v" if os.environ.get("CT_PTXAS_VERBOSE") else "-O3",
               *common, "-c", str(path), "-o", str(obj)]
    else:
        cmd = [nvcc(), "-x", "c++", *common, "-c", str(path), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if os.environ.get("CT_PTXAS_VERBOSE"):
        sys.stderr.write(res.stderr)


def stale() -> bool:
    if not LIB.exists():
        return True
    built = LIB.stat().st_mtime
    deps = [HERE / f for f in SOURCES + HEADERS if (HERE / f).exists()] + [pathlib.Path(__file__)]
    return any(p.stat().st_mtime > built for p in deps)


def build(force: bool = False) -> pathlib.Path:
    if not force and not stale():
        return LIB
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    objs = [OUT_DIR / (pathlib.Path(s).stem + ".o") for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(lambda a: _compile(*a), zip(SOURCES, objs)))
    tmp = OUT_DIR / (LIB.name + ".tmp")
    cmd = [nvcc(), ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
