"""Build the CUDA library (sm_103a) and the C++ command-line driver in place.

    python -m turbulent_lbm_multigpu_gb300.build

Produces, next to this file:
  liblbm_gb300.so   the C ABI of include/lbm_gb300.h
  lbm_gb300         the C++ driver (include/lbm_gb300/*.hpp over the C ABI)

Every kernel is compiled for sm_103a only, with -fmad=false so that no
multiply-add is contracted (results are bit-identical to the reference
kernels' arithmetic) and with IEEE division and square root.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB = PKG / "liblbm_gb300.so"
CLI = PKG / "lbm_gb300"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
           "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]

CU_SOURCES = ["lbm_capi.cu", "lbm_batch.cu", "lbm_io.cu", "lbm_f64fma.cu"]
# the contracted FP64 kernels: products may fuse into sums in this unit only
FMAD_SOURCES = {"lbm_f64fma.cu"}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise FileNotFoundError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")
    return exe


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _deps():
    return [p for p in list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.rglob("*.h*"))
            + [Path(__file__)]]


def build_lib(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale(LIB, _deps()):
        return LIB
    objdir = PKG / "_build"
    objdir.mkdir(exist_ok=True)

    def compile_one(src):
        obj = objdir / (Path(src).stem + ".o")
        flags = [("-fmad=true" if f == "-fmad=false" and src in FMAD_SOURCES else f) for f in NVFLAGS]
        cmd = [nvcc()] + ARCH + flags + ["-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        subprocess.run(cmd, check=True)
        return str(obj)

    with ThreadPoolExecutor(max(1, len(CU_SOURCES))) as ex:
        objs = list(ex.map(compile_one, CU_SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + objs + ["-lcudart"], check=True)
    tmp.replace(LIB)
    return LIB


def build_cli(force: bool = False) -> Path | None:
    src = CSRC / "lbm_main.cpp"
    if not src.exists():
        return None
    if not force and not _stale(CLI, _deps() + [src, LIB]):
        return CLI
    cuda_home = Path(nvcc()).resolve().parent.parent
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{cuda_home / 'include'}",
           str(src), "-o", str(CLI), f"-L{PKG}", "-llbm_gb300", f"-Wl,-rpath,{PKG}",
           f"-L{cuda_home / 'lib64'}", "-lcudart", f"-Wl,-rpath,{cuda_home / 'lib64'}"]
    subprocess.run(cmd, check=True)
    return CLI


def build(force: bool = False, verbose: bool = False) -> Path:
    lib = build_lib(force, verbose)
    build_cli(force)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
