"""Weak and strong scaling sweeps over decompositions of one domain on one GPU.

    python -m turbulent_lbm_multigpu_gb300.scaling strong [--size 256 256 256] [--exp 3] [--steps 200]
    python -m turbulent_lbm_multigpu_gb300.scaling weak [--sub 128 128 128] [--exp 3] [--steps 200]

The reference's benchmark.py launches one MPI rank per subdomain and each
run appends its timing to output/benchmark/benchmark_<NP>.ini
(src/CController.hpp:445-477); analyse() averages the experiments of every
file.  Here every decomposition runs in this process on one GPU (all
subdomains resident, device-local halo exchanges) through the domain API,
and the records keep the reference's layout: sections [EXPn] with NP and
CUBE_X, CUBE_Y, CUBE_Z, SECONDS, FPS, MLUPS, BANDWIDTH.  Strong scaling keeps
the domain fixed and splits it further; weak scaling keeps the subdomain
fixed and grows the domain with the number of subdomains.  The lattice is
the reference-derived cavity (BGK + Smagorinsky, lid 0.1, Re 1e4), f32 unless
--storage says otherwise.
"""
from __future__ import annotations

import argparse
import configparser
import json
import time
from pathlib import Path

KEYS = ("CUBE_X", "CUBE_Y", "CUBE_Z", "SECONDS", "FPS", "MLUPS", "BANDWIDTH")
DECOMPOSITIONS = ((1, 1, 1), (2, 1, 1), (2, 2, 1), (2, 2, 2), (4, 2, 2), (4, 4, 2))


def append_record(path: Path, exp: int, np_: int, cube, seconds: float, loops: int, bytes_per_value: int,
                  vis: bool = False):
    """One run in the reference's record layout (FPS = loops / seconds,
    MLUPS over the whole cube, BANDWIDTH = MLUPS x (2*19 + 1 (+3)) x value bytes)."""
    fps = loops / seconds
    mlups = fps * cube[0] * cube[1] * cube[2] * 1e-6
    floats = 19.0 * 2.0 + 1.0 + (3.0 if vis else 0.0)
    path.parent.mkdir(parents=True, exist_ok=True)
    with open(path, "a") as f:
        f.write(f"[EXP{exp}]\nNP : {np_}\n")
        f.write(f"CUBE_X : {cube[0]}\nCUBE_Y : {cube[1]}\nCUBE_Z : {cube[2]}\n")
        f.write(f"SECONDS : {seconds!r}\nFPS : {fps!r}\nMLUPS : {mlups!r}\nBANDWIDTH : {mlups * floats * bytes_per_value!r}\n\n")


def analyse(filenames):
    """Average every key over the experiments of each file, keyed by NP (the
    reference's benchmark.py analyse())."""
    out = {}
    for name in filenames:
        cfg = configparser.ConfigParser()
        cfg.read(name)
        secs = [s for s in cfg.sections() if s.startswith("EXP")]
        if not secs:
            continue
        np_ = cfg.getint(secs[0], "NP")
        out[np_] = {k: sum(cfg.getfloat(s, k) for s in secs) / len(secs) for k in KEYS if cfg.has_option(secs[0], k)}
    return out


def _params(api, storage, length):
    import numpy as np

    rdt = np.float64 if storage == api.F64 else np.float32
    tau = rdt(3.0 * 0.1 * length / 1e4 + 0.5)
    return api.Params.make(float(rdt(1) / tau), float(tau), api.les_coefficient(0.17), (0.0, 0.0, 0.0), 0.1)


def run_one(api, size, nums, storage, steps, warmup=10):
    """Seconds for `steps` steps of the domain (CUDA graph replay, synchronised)."""
    D = api.Domain(size, nums, storage, store_velocity=False, store_density=False)
    D.set_params(_params(api, storage, size[0]))
    D.set_halo_mode(1)
    D.reset()
    D.perturb(1234, 1e-3)
    D.run(warmup)
    api.check(api.lib().lbm_cu_synchronize(None))
    t0 = time.perf_counter()
    D.run(steps)
    api.check(api.lib().lbm_cu_synchronize(None))
    return time.perf_counter() - t0


def sweep(kind, size=(256, 256, 256), sub=(128, 128, 128), exps=3, steps=200, storage="f32",
          outdir="output/benchmark", decompositions=DECOMPOSITIONS):
    from . import build, capi as api

    build.build()
    st = api.STORAGE_NAMES[storage]
    files = []
    for nums in decompositions:
        cube = tuple(size) if kind == "strong" else tuple(s * n for s, n in zip(sub, nums))
        if any(c % n for c, n in zip(cube, nums)):
            continue
        np_ = nums[0] * nums[1] * nums[2]
        path = Path(outdir) / f"benchmark_{np_}.ini"
        if path.exists():
            path.unlink()
        for e in range(1, exps + 1):
            append_record(path, e, np_, cube, run_one(api, cube, nums, st, steps), steps,
                          {"f32": 4, "f64": 8}.get(storage, 2))
        files.append(str(path))
    return analyse(files)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("kind", choices=["strong", "weak"])
    ap.add_argument("--size", type=int, nargs=3, default=[256, 256, 256])
    ap.add_argument("--sub", type=int, nargs=3, default=[128, 128, 128])
    ap.add_argument("--exp", type=int, default=3)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--storage", default="f32", choices=["f32", "f64", "f16", "bf16"])
    ap.add_argument("--out", default="output/benchmark")
    a = ap.parse_args()
    res = sweep(a.kind, a.size, a.sub, a.exp, a.steps, a.storage, a.out)
    base = res.get(1)
    for r in res.values():
        # all subdomains share one GPU: the ratio to the undecomposed run is
        # the cost of the decomposition (ghost layers and halo exchanges)
        if base:
            r["MLUPS_VS_NP1"] = r["MLUPS"] / base["MLUPS"]
    print(json.dumps({"kind": a.kind, "storage": a.storage, "results": {str(k): v for k, v in sorted(res.items())}}))


if __name__ == "__main__":
    main()
