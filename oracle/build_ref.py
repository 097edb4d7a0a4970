"""Recipe that compiles the reference's own OpenCL kernels as C++.

TEST INFRASTRUCTURE ONLY (part of the oracle).  The four kernel files
(src/cl_programs/{lbm_init,lbm_alpha,lbm_beta,copy_buffer_rect}.cl) are
compiled in place from the reference tree -- nothing is copied -- together
with oracle/ref_shim (our keyword shim and work-group emulator) and a
definition prefix equal to the one the reference host generates at run time
(src/CLbmSolver.hpp:319-373, plus LOCAL_WORK_GROUP_SIZE from :419-422).
Sizes are compile-time macros in the reference (DOMAIN_CELLS_X/Y/Z), so each
(T, X, Y, Z, work-group size) gets its own shared library under oracle/_ref/.

The reference tree exists only on the development machine; on a machine
without it, `available()` is False and callers skip the reference pin.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SHIM = HERE / "ref_shim"
# the reference tree: LBM_REF_DIR, else a directory named "reference" beside
# this repository's root
REF_DIR = Path(os.environ.get("LBM_REF_DIR") or (HERE.parent.parent / "reference"))

KINDS = {"lbm_init": 1, "lbm_alpha": 2, "lbm_beta": 3, "copy_buffer_rect": 4}

# flags: src/CLbmSolver.hpp:30-33
FLAGS = {"FLAG_OBSTACLE": 1, "FLAG_FLUID": 2, "FLAG_VELOCITY_INJECTION": 4, "FLAG_GHOST_LAYER": 8}


def available() -> bool:
    return all((REF_DIR / "src" / "cl_programs" / f"{k}.cl").is_file() for k in KINDS)


def _prefix(dtype: str, nx: int, ny: int, nz: int, wg: int) -> str:
    t = "float" if dtype == "f32" else "double"
    size = 4 if dtype == "f32" else 8
    lines = [
        f"#define SIZE_DD_HOST_BYTES ({19 * size})",
        f"typedef {t} T;",
        f"typedef {t}2 T2;",
        f"typedef {t}4 T4;",
        f"typedef {t}8 T8;",
        f"typedef {t}16 T16;",
        f"#define DOMAIN_CELLS_X\t({nx})",
        f"#define DOMAIN_CELLS_Y\t({ny})",
        f"#define DOMAIN_CELLS_Z\t({nz})",
        "#define GLOBAL_WORK_GROUP_SIZE\t(DOMAIN_CELLS_X*DOMAIN_CELLS_Y*DOMAIN_CELLS_Z)",
    ]
    lines += [f"#define {k}\t({v})" for k, v in FLAGS.items()]
    lines += ["#define STORE_VELOCITY 1", "#define STORE_DENSITY 1", f"#define LOCAL_WORK_GROUP_SIZE\t({wg})"]
    return "\n".join(lines) + "\n"


def lib_path(dtype: str, nx: int, ny: int, nz: int, wg: int = 128) -> Path:
    return OUT / f"ref_{dtype}_{nx}x{ny}x{nz}_wg{wg}.so"


def build(dtype: str, nx: int, ny: int, nz: int, wg: int = 128, force: bool = False) -> Path:
    """Compile the reference kernels for one configuration; returns the .so path."""
    if dtype not in ("f32", "f64"):
        raise ValueError("the reference kernels exist in float and double only")
    if not available():
        raise FileNotFoundError(f"reference kernel sources not found under {REF_DIR}")
    so = lib_path(dtype, nx, ny, nz, wg)
    if so.exists() and not force:
        return so
    work = OUT / so.stem
    work.mkdir(parents=True, exist_ok=True)
    prefix = work / "prefix.h"
    prefix.write_text(_prefix(dtype, nx, ny, nz, wg))
    cxx = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-w",
           f"-I{REF_DIR}", f"-I{SHIM}"]

    def compile_one(item):
        name, kind = item
        obj = work / f"{name}.o"
        cmd = cxx + [f'-DREF_PREFIX="{prefix}"', f'-DREF_SOURCE="{REF_DIR / "src/cl_programs" / (name + ".cl")}"',
                     f"-DREF_KIND={kind}", "-c", str(SHIM / "ref_kernel.cpp"), "-o", str(obj)]
        subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(4) as ex:
        objs = list(ex.map(compile_one, KINDS.items()))
    tmp = so.with_suffix(".so.tmp")
    subprocess.run(["g++", "-shared", "-fopenmp", "-o", str(tmp)] + [str(o) for o in objs], check=True)
    tmp.replace(so)
    return so


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--dtype", default="f32")
    ap.add_argument("--size", type=int, nargs=3, default=[64, 64, 64])
    ap.add_argument("--wg", type=int, default=128)
    a = ap.parse_args()
    print(build(a.dtype, *a.size, a.wg, force=True))
