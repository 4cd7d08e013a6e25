"""Builds libcaustic_gb300.so for sm_103a into caustic-tracer_gb300/_build/,
and beside it the Node-API addon caustic_addon.node (napi/caustic_addon.c),
linked against the library with an $ORIGIN run path.

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
ADDON = OUT_DIR / "caustic_addon.node"
NAPI = PKG / "napi"
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


def addon_stale() -> bool:
    if not ADDON.exists():
        return True
    built = ADDON.stat().st_mtime
    deps = [LIB, NAPI / "caustic_addon.c", NAPI / "node_api_min.h", PKG.parent / "include" / "caustic.h"]
    return any(p.stat().st_mtime > built for p in deps)


def build_addon(force: bool = False) -> pathlib.Path:
    """The Node-API addon: plain C (gcc), Node-API symbols left for Node to provide at load time."""
    if not force and not addon_stale():
        return ADDON
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler (gcc) found for the Node-API addon")
    tmp = OUT_DIR / (ADDON.name + ".tmp")
    cmd = [cc, "-std=c11", "-O2", "-fPIC", "-shared", "-Wall", "-Wextra", "-Werror", f"-I{NAPI}",
           f"-I{PKG.parent / 'include'}", str(NAPI / "caustic_addon.c"), "-o", str(tmp), f"-L{OUT_DIR}",
           "-lcaustic_gb300", "-Wl,-rpath,$ORIGIN", "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compiling the Node-API addon failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, ADDON)
    return ADDON


def build(force: bool = False) -> pathlib.Path:
    if not force and not stale():
        build_addon()
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
    build_addon(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
