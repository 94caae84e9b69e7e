"""Builds the reference MPLA for parity checks: oracle/_ref/libmplaref.so.

TEST INFRASTRUCTURE.  The reference's hot-path sources are compiled as they
are (no edit) with a single-rank MPI stand-in (oracle/ref_mpi/mpi.h) and our
harness (oracle/ref_harness.cu), which drives them through their public API.

Steps
  1. stage: where the reference tree is present (the x86 development
     machine), copy the nine source files of the path into oracle/_ref/src/.
     That folder is git-ignored (never committed) but travels with the
     working tree to the AArch64 machine that runs the GPU work, where an x86
     build cannot run and the reference tree is absent, so the sources are
     compiled there.
  2. compile: g++ for mpla.cpp (host code), nvcc for the CUDA files
     (relocatable device code for the virtual system_assembler, device-linked
     like the reference's own Makefile:96-114), one -gencode for sm_103a.
     cudaThreadSynchronize, removed in CUDA 13, is mapped to
     cudaDeviceSynchronize; stdio.h and math.h are force-included because the
     sources rely on transitive includes.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
# Source tree of the reference (its src/ folder): MPLA_REFERENCE_SRC when set,
# else where the development machine mounts it.  Only stage() reads it.
REF_TREE = Path(os.environ.get("MPLA_REFERENCE_SRC", "/root/reference/src"))
OUT = HERE / "_ref"
SRC = OUT / "src"
LIB = OUT / "libmplaref.so"
FILES = ["mpla.cpp", "mpla.h", "kernel.cu", "kernel.h", "generic_system_adapter.cu", "generic_system_adapter.h",
         "kernel_system_assembler.cu", "kernel_system_assembler.h", "system_assembler.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMPAT = ["-DcudaThreadSynchronize=cudaDeviceSynchronize", "-include", "stdio.h", "-include", "math.h"]


def stage(ref_tree: Path | None = None) -> bool:
    """Copies the path's sources from `ref_tree` (default REF_TREE) into
    oracle/_ref/src; True when the staged sources are complete."""
    tree = Path(ref_tree) if ref_tree else REF_TREE
    if not tree.is_dir():
        return all((SRC / f).exists() for f in FILES)
    SRC.mkdir(parents=True, exist_ok=True)
    for f in FILES:
        dst = SRC / f
        if dst.exists():
            os.chmod(dst, 0o644)
        shutil.copyfile(tree / f, dst)
        os.chmod(dst, 0o644)
    return True


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + res.stdout + res.stderr)


def build(ref_tree: Path | None = None) -> Path:
    if not stage(ref_tree):
        raise RuntimeError("reference sources not staged (oracle/_ref/src) and no reference tree to stage from")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda = Path(nvcc).resolve().parent.parent
    obj = OUT / "obj"
    obj.mkdir(parents=True, exist_ok=True)
    deps = [SRC / f for f in FILES] + [HERE / "ref_harness.cu", HERE / "ref_mpi" / "mpi.h", Path(__file__)]
    if LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    inc = ["-I", str(HERE / "ref_mpi"), "-I", str(SRC)]
    cxx = shutil.which("g++") or "g++"
    _run([cxx, "-O3", "-fPIC", "-std=c++14", *inc, "-I", str(cuda / "include"), *COMPAT, "-c",
          str(SRC / "mpla.cpp"), "-o", str(obj / "mpla.o")])
    common = [nvcc, *ARCH, "-O3", "-Xcompiler", "-fPIC", *inc, *COMPAT]
    _run([*common, "-c", str(SRC / "kernel.cu"), "-o", str(obj / "kernel.o")])
    for name in ["generic_system_adapter", "kernel_system_assembler"]:
        _run([*common, "-dc", str(SRC / f"{name}.cu"), "-o", str(obj / f"{name}.o")])
    _run([*common, "-dc", str(HERE / "ref_harness.cu"), "-o", str(obj / "ref_harness.o")])
    objs = [str(obj / f) for f in ["mpla.o", "kernel.o", "generic_system_adapter.o", "kernel_system_assembler.o",
                                   "ref_harness.o"]]
    _run([nvcc, *ARCH, "-shared", "-Xlinker", "-Bsymbolic", "-o", str(LIB), *objs, "-lcublas", "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build())
