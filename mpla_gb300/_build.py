"""Build recipe of the native library (libmpla.so) for GB300 (sm_103a).

Every translation unit under ``csrc/`` is compiled by nvcc in parallel into
``_build/`` and linked into ``lib/libmpla.so``, which exports both the mpla.h
drop-in API (C++ linkage) and the C ABI of ``include/mpla_gb300.h``.
``csrc_device/generic_device.cu`` becomes ``lib/mpla_generic_device.o``
(relocatable device code): users device-link it into the module that defines
their system_assembler subclasses.  No
cmake, one ``-gencode``, object files rebuilt only when a source or header is
newer, so a fresh build takes about a minute and a rebuild seconds.
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
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libmpla.so"
DEVICE_SRC = PKG / "csrc_device" / "generic_device.cu"
DEVICE_OBJ = LIBDIR / "mpla_generic_device.o"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE), "-I", str(CSRC)]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmpla.so")
    return cand


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, extra: list[str]) -> Path:
    obj = BUILD / (src.stem + ".o")
    deps = [src] + _headers()
    if _stale(obj, deps):
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def _compile_device(extra: list[str]) -> Path:
    if _stale(DEVICE_OBJ, [DEVICE_SRC] + _headers()):
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-rdc=true", "-c", str(DEVICE_SRC), "-o", str(DEVICE_OBJ)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {DEVICE_SRC.name}:\n{res.stdout}\n{res.stderr}")
    return DEVICE_OBJ


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile csrc/*.cu and link lib/libmpla.so; returns the library path."""
    extra = list(extra or [])
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    workers = min(len(sources) + 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        dev = ex.submit(_compile_device, extra)
        objs = list(ex.map(lambda s: _compile(s, extra), sources))
        dev.result()
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcublas", "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
