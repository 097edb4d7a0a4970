"""Generate the golden fixtures from the reference's own kernels.

Run on a machine that has the reference tree (LBM_REF_DIR, default: the
directory `reference` beside this repository):  python tests/golden/make_golden.py

The reference kernels (src/cl_programs/*.cl) are compiled as C++ by
oracle/build_ref.py and driven by the host logic of oracle/oracle.py.  The
fixtures pin the C oracle and the CUDA path on machines where the reference
tree is absent:
  cavity_<T>_12x8x8.npz   full arrays (populations, velocity, density,
                           flags) at selected steps of a perturbed lid cavity
                           with gravity, T = f32 and f64;
  hashes.json              per-step SHA-256 of the fluid and lid cells'
                           populations, velocity and density for the 64^3
                           lid cavity (Re 1000, U 0.05, f32 and f64) and for
                           a 2x2x1 decomposition.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import oracle as O  # noqa: E402

SEED = 1234


def state_hash(lat) -> str:
    """SHA-256 of the wrap-independent state: every population, velocity and
    density value of the fluid and lid cells, plus all flags."""
    m = O.fluid_mask(lat.flags)
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(lat.dd[:, m]).tobytes())
    h.update(np.ascontiguousarray(lat.vel[:, m]).tobytes())
    h.update(np.ascontiguousarray(lat.rho[m]).tobytes())
    h.update(np.ascontiguousarray(lat.flags).tobytes())
    return h.hexdigest()


def small_case(storage):
    dims = (12, 8, 8)
    rdt = O.STORAGE[storage][1]
    p = O.Params.lattice(O.cavity_tau(0.05, dims[0], 100.0), 0.05, dtype=rdt,
                         gravity=tuple(float(rdt(g)) for g in (1e-5, -2e-5, 3e-6)))
    return dims, p


def c1_case(storage):
    rdt = O.STORAGE[storage][1]
    return (64, 64, 64), O.Params.lattice(O.cavity_tau(0.05, 64, 1000.0), 0.05, dtype=rdt)


def decomposed_case():
    p = O.Params.lattice(O.cavity_tau(0.1, 22, 1000.0), 0.1, dtype=np.float32)
    return (24, 16, 16), (2, 2, 1), p


def main():
    out = {}
    for st in ("f32", "f64"):
        dims, p = small_case(st)
        s = O.single(O.RefKernels(st, *dims), dims, p, st)
        s.k.perturb(s.lat, (0, 0, 0), dims, SEED, 1e-2)
        arrays = {"dd0": s.lat.dd.copy(), "flags": s.lat.flags.copy()}
        for k in range(1, 9):
            s.step()
            if k in (1, 2, 3, 8):
                arrays[f"dd{k}"] = s.lat.dd.copy()
                arrays[f"vel{k}"] = s.lat.vel.copy()
                arrays[f"rho{k}"] = s.lat.rho.copy()
        np.savez_compressed(HERE / f"cavity_{st}_12x8x8.npz", **arrays)

    for st, steps in (("f32", 100), ("f64", 40)):
        dims, p = c1_case(st)
        s = O.single(O.RefKernels(st, *dims), dims, p, st)
        out[f"c1_{st}"] = [state_hash(s.lat)]
        for _ in range(steps):
            s.step()
            out[f"c1_{st}"].append(state_hash(s.lat))

    size, nums, p = decomposed_case()
    D = O.Domain(lambda d: O.RefKernels("f32", *d), size, nums, p, "f32")
    D.perturb(SEED, 1e-2)
    out["decomposed_f32"] = []
    for _ in range(24):
        D.step()
        out["decomposed_f32"].append([state_hash(sol.lat) for _, sol, _ in D.parts])
    (HERE / "hashes.json").write_text(json.dumps(out, indent=0))


if __name__ == "__main__":
    main()
