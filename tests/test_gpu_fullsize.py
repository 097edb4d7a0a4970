"""Parity at the sizes the benchmark runs: the CUDA path against the oracle.

The benchmark's cavity (256^3 cells in 2x2x1 subdomains of 128x128x256 on one
GPU, D3Q19 BGK + Smagorinsky Cs 0.17, Re 10^4, lid 0.1, seeded start-up
+-1e-3) is run for 20 steps through the domain's step and halo launches --
the exchange of src/CController.hpp:265-391 over the CComm geometry of
src/CManager.hpp:78-204 -- and every subdomain's populations, velocity,
density and flags are compared with the oracle's decomposed run after each
step, bit for bit.  Steps 13-20 replay the captured graph, as the benchmark
does.  The single 512^3 lattices (the benchmark's extra sizes) have more than
2^31 population elements, so their plane offsets need 64-bit arithmetic; they
are compared with the oracle for four steps.

Bar: bit equality.  The tolerances of the parity tests (population
max-relative error 1e-6 in f32 and 1e-12 in f64) are asserted on any
difference before the equality is.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import bits, max_rel

pytestmark = pytest.mark.gpu

SEED, AMP = 1234, 1e-3
U_LID, RE, CS = 0.1, 1e4, 0.17
TOL = {"f32": 1e-6, "f64": 1e-12, "f16": 1e-6, "bf16": 1e-6, "c16": 1e-6}


def same(a, b) -> bool:
    return a.shape == b.shape and np.array_equal(bits(a), bits(b))


def params(api, O, storage, edge):
    rdt = O.STORAGE[storage][1]
    p = O.Params.lattice(O.cavity_tau(U_LID, edge, RE), U_LID, CS, dtype=rdt)
    return p, api.Params.make(p.inv_tau, p.tau0, p.les_c, p.gravity, p.lid, p.gravity_mode)


def check_lattice(api, L, sol, storage, where, fields=True, slab=64):
    """Populations slab by slab of z planes (bounded host memory at 512^3),
    then flags, velocity and density."""
    nx, ny, nz = L.dims
    for z0 in range(0, nz, slab):
        dz = min(slab, nz - z0)
        got = L.read(api.FIELD_DD, origin=(0, 0, z0), size=(nx, ny, dz))
        raw = sol.lat.dd[:, z0:z0 + dz]
        want = raw if storage in ("f32", "f64") else sol.k.decode(raw)
        if not same(got, want):
            err = max_rel(got, want)
            assert err <= TOL[storage], f"populations {where}, z {z0}..{z0 + dz - 1}: max rel {err:.3g}"
            raise AssertionError(f"populations {where}, z {z0}..{z0 + dz - 1}: "
                                 f"{int((bits(got) != bits(want)).sum())} elements differ (max rel {err:.3g})")
    if not fields:
        return
    assert same(L.read(api.FIELD_FLAGS)[0], sol.lat.flags), f"flags {where}"
    assert same(L.read(api.FIELD_VELOCITY), sol.lat.vel), f"velocity {where}"
    assert same(L.read(api.FIELD_DENSITY)[0], sol.lat.rho), f"density {where}"


@pytest.mark.parametrize("storage,halo_mode", [("f32", 0), ("f32", 1), ("f64", 1), ("f64", 0), ("f16", 1),
                                               ("bf16", 0), ("c16", 1)])
def test_cavity_256cube_2x2x1_matches_oracle(capi, oracle_mod, storage, halo_mode):
    api, O = capi, oracle_mod
    size, nums = (256, 256, 256), (2, 2, 1)
    p, gp = params(api, O, storage, size[0])
    D = api.Domain(size, nums, api.STORAGE_NAMES[storage], True, True)
    D.set_params(gp)
    D.set_halo_mode(halo_mode)
    D.reset()
    D.perturb(SEED, AMP)
    R = O.Domain(lambda d: O.OracleKernels(storage), size, nums, p, storage, halo_mode=halo_mode)
    R.perturb(SEED, AMP)
    assert D.sub == (128, 128, 256)
    for L, (_, s, _) in zip(D.subdomains, R.parts):
        check_lattice(api, L, s, storage, "after start-up")
    for _ in range(12):  # eager steps, velocity and density written every step
        D.run(1, use_graph=False)
        R.step()
        for L, (_, s, _) in zip(D.subdomains, R.parts):
            check_lattice(api, L, s, storage, f"after step {R.counter}")
    D.set_store_interval(0)  # pairs replay the graph, the last step of a call stores u and rho
    for _ in range(2):
        D.run(4, use_graph=True)
        for _ in range(4):
            R.step()
        assert D.counter == R.counter
        for L, (_, s, _) in zip(D.subdomains, R.parts):
            check_lattice(api, L, s, storage, f"after step {R.counter} (graph replay)")


@pytest.mark.parametrize("storage", ["f32", "f16", "c16"])
def test_lattice_512cube_matches_oracle(capi, oracle_mod, storage):
    """One 512^3 lattice (19 x 134M population elements: 64-bit plane
    offsets), the benchmark's default kernel shape, four steps."""
    api, O = capi, oracle_mod
    dims = (512, 512, 512)
    p, gp = params(api, O, storage, dims[0])
    p.store_vel = p.store_rho = False
    L = api.Lattice(*dims, api.STORAGE_NAMES[storage], False, False)
    L.set_params(gp)
    L.init([api.FLAG_OBSTACLE] * 6)
    nx, ny, nz = dims
    L.write(api.FIELD_FLAGS, np.full((nz - 2) * (nx - 2), api.FLAG_VELOCITY_INJECTION, np.int32),
            origin=(1, ny - 2, 1), size=(nx - 2, 1, nz - 2))
    L.perturb((0, 0, 0), dims, SEED, AMP)
    s = O.single(O.OracleKernels(storage), dims, p, storage)
    s.k.perturb(s.lat, (0, 0, 0), dims, SEED, AMP)
    for k in range(4):
        L.step(s.lat.counter & 1)
        s.step()
        check_lattice(api, L, s, storage, f"after step {k + 1}", fields=False)
