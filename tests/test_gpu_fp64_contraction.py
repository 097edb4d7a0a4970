"""Double storage with contracted FP64 kernels against the bit-exact oracle.

lbm_cu_set_fp64_contraction lets the double step kernels fuse products into
sums (one rounding instead of two).  Their results are no longer bit-equal
to the reference arithmetic; the bound is the FP64 parity tolerance,
population max-relative error <= 1e-12 per step.  Two checks:
  * per step: each step starts from the oracle's state (uploaded), so the
    difference after it is that step's own error;
  * accumulated: a free run of 20 steps stays within the same bound.
The bit-exact kernels stay the default and keep bit equality (checked last).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import max_rel, n_diff

pytestmark = pytest.mark.gpu

SEED = 1234
TOL = 1e-12


def cavity(api, O, dims, cs, re, u, amp):
    p = O.Params.lattice(O.cavity_tau(u, dims[0], re), u, cs, dtype=np.float64)
    L = api.Lattice(*dims, api.F64, True, True)
    L.set_params(api.Params.make(p.inv_tau, p.tau0, p.les_c, p.gravity, p.lid))
    L.init([api.FLAG_OBSTACLE] * 6)
    nx, ny, nz = dims
    L.write(api.FIELD_FLAGS, np.full((nz - 2) * (nx - 2), api.FLAG_VELOCITY_INJECTION, np.int32),
            origin=(1, ny - 2, 1), size=(nx - 2, 1, nz - 2))
    L.perturb((0, 0, 0), dims, SEED, amp)
    s = O.single(O.OracleKernels("f64"), dims, p, "f64")
    s.k.perturb(s.lat, (0, 0, 0), dims, SEED, amp)
    return L, s


@pytest.mark.parametrize("cs", [0.0, 0.17])
def test_contracted_step_error_per_step(capi, oracle_mod, cs):
    """64^3 lid cavity (config-1 geometry), Re 1000, lid 0.05."""
    api, O = capi, oracle_mod
    L, s = cavity(api, O, (64, 64, 64), cs, 1000.0, 0.05, 1e-2)
    L.set_fp64_contraction(True)
    worst, changed = 0.0, 0
    for k in range(20):
        L.write(api.FIELD_DD, s.lat.dd)  # start the step from the oracle's state
        L.step(s.lat.counter & 1)
        s.step()
        got = L.read(api.FIELD_DD)
        err = max_rel(got, s.lat.dd)
        assert err <= TOL, f"step {k + 1}: max rel {err:.3g}"
        worst = max(worst, err)
        changed += n_diff(got, s.lat.dd)
    assert changed > 0, "the contracted kernels ran the bit-exact arithmetic"


def test_contracted_free_run(capi, oracle_mod):
    api, O = capi, oracle_mod
    L, s = cavity(api, O, (48, 40, 36), 0.17, 5000.0, 0.1, 1e-2)
    L.set_fp64_contraction(True)
    for k in range(20):
        L.step(s.lat.counter & 1)
        s.step()
        err = max_rel(L.read(api.FIELD_DD), s.lat.dd)
        assert err <= TOL, f"step {k + 1}: max rel {err:.3g}"
    L.set_fp64_contraction(False)  # back to the bit-exact kernels: equal from the oracle's state on
    L.write(api.FIELD_DD, s.lat.dd)
    for _ in range(4):
        L.step(s.lat.counter & 1)
        s.step()
        assert n_diff(L.read(api.FIELD_DD), s.lat.dd) == 0


def test_contracted_domain_256cube(capi, oracle_mod):
    """The benchmark's decomposition (256^3 in 2x2x1, Re 10^4, lid 0.1, Cs
    0.17) with contracted kernels: 10 steps within the bound."""
    api, O = capi, oracle_mod
    size, nums = (256, 256, 256), (2, 2, 1)
    p = O.Params.lattice(O.cavity_tau(0.1, 256, 1e4), 0.1, 0.17, dtype=np.float64)
    D = api.Domain(size, nums, api.F64, False, False)
    D.set_params(api.Params.make(p.inv_tau, p.tau0, p.les_c, p.gravity, p.lid))
    D.set_fp64_contraction(True)
    D.reset()
    D.perturb(SEED, 1e-3)
    R = O.Domain(lambda d: O.OracleKernels("f64"), size, nums, p, "f64", halo_mode=0)
    R.perturb(SEED, 1e-3)
    for _ in range(5):
        D.run(2, use_graph=True)
        R.step()
        R.step()
        for L, (_, sol, _) in zip(D.subdomains, R.parts):
            err = max_rel(L.read(api.FIELD_DD), sol.lat.dd)
            assert err <= TOL, f"step {R.counter}: max rel {err:.3g}"


def test_contraction_needs_double(capi):
    api = capi
    L = api.Lattice(8, 8, 8, api.F32, False, False)
    with pytest.raises(api.LbmError, match="double storage only"):
        L.set_fp64_contraction(True)
