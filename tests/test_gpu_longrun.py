"""The check for long runs, where trajectories of different precisions
separate: after 3000 steps of a lid-driven cavity with the subgrid model,
shifted half storage keeps the FP64 run's velocity statistics, centreline
profile and kinetic energy within 1 %."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_half_storage_keeps_fp64_statistics_over_a_long_run(capi):
    from turbulent_lbm_multigpu_gb300 import experiments as ex

    api = capi
    dims, re, lid, cs, steps = (96, 96, 96), 5000.0, 0.1, 0.17, 3000
    tau = ex.tau_for(lid, float(dims[0]), re)
    layout = (steps - 1) & 1  # the last step was an alpha step: opposite slots
    runs = {}
    for st in (api.F64, api.F16):
        L = ex.cavity_lattice(dims, st, tau, cs, lid, 1234, 1e-3, store_velocity=True)
        L.run(0, steps)
        api.synchronize()
        u = L.read(api.FIELD_VELOCITY).astype(np.float64)
        fluid = L.read(api.FIELD_FLAGS)[0] == api.FLAG_FLUID
        speed = np.sqrt((u ** 2).sum(axis=0))[fluid]
        runs[st] = {"mean": speed.mean(), "rms": np.sqrt((speed ** 2).mean()),
                    "ke": L.reduce_conserved(layout)[4], "line": ex.centerline_ux(L, layout)}
    ref, half = runs[api.F64], runs[api.F16]
    assert abs(half["mean"] / ref["mean"] - 1) < 0.01
    assert abs(half["rms"] / ref["rms"] - 1) < 0.01
    assert abs(half["ke"] / ref["ke"] - 1) < 0.01
    assert np.abs(half["line"] - ref["line"]).max() < 0.01 * np.abs(ref["line"]).max()
