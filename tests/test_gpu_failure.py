"""The failure path of the staged kernels' bounded barrier waits, checked
without a fault: a check kernel's wait on a barrier that nothing completes
runs out, the host reports it once, and the device keeps computing the
same results."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import n_diff

pytestmark = pytest.mark.gpu


def test_bounded_wait_timeout_is_reported_and_cleared(capi, oracle_mod):
    api, O = capi, oracle_mod
    api.synchronize()
    with pytest.raises(api.LbmError, match="polls"):
        api.check_wait_timeout(0)
    api.check_wait_timeout(1 << 12)
    with pytest.raises(api.LbmError, match="gave up waiting"):
        api.synchronize()
    api.synchronize()  # reported once, then cleared

    # the staged kernels still agree with the oracle bit for bit afterwards
    dims = (32, 20, 16)
    nx, ny, nz = dims
    p = O.Params.lattice(O.cavity_tau(0.05, nx, 1000.0), 0.05, 0.17, dtype=np.float32)
    L = api.Lattice(*dims, api.F16, True, True)
    L.set_params(api.Params.make(p.inv_tau, p.tau0, p.les_c, p.gravity, p.lid))
    L.init([api.FLAG_OBSTACLE] * 6)
    L.write(api.FIELD_FLAGS, np.full((nz - 2) * (nx - 2), api.FLAG_VELOCITY_INJECTION, np.int32),
            origin=(1, ny - 2, 1), size=(nx - 2, 1, nz - 2))
    L.perturb((0, 0, 0), dims, 99, 1e-2)
    s = O.single(O.OracleKernels("f16"), dims, p, "f16")
    s.k.perturb(s.lat, (0, 0, 0), dims, 99, 1e-2)
    for k in range(4):
        L.step(k & 1)
        s.step()
    api.synchronize()
    assert n_diff(L.read(api.FIELD_DD), s.k.decode(s.lat.dd)) == 0
