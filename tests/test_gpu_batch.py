"""Ensembles and the solve server: every cavity's result equals the same
cavity run alone, bit for bit, whatever else shares its launches."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import n_diff

pytestmark = pytest.mark.gpu


def lone(api, c):
    """The cavity of `c` run alone on its own lattice, one launch per step."""
    L = api.Lattice(c.nx, c.ny, c.nz, c.storage, True, False)
    tau = np.float64(c.tau0) if c.storage == api.F64 else np.float32(c.tau0)
    inv = float(1.0 / tau) if c.storage == api.F64 else float(np.float32(1) / tau)
    L.set_params(api.Params.make(inv, float(tau), api.les_coefficient(c.cs), (0, 0, 0), c.lid))
    L.init([api.FLAG_OBSTACLE] * 6)
    L.write(api.FIELD_FLAGS, np.full((c.nz - 2) * (c.nx - 2), api.FLAG_VELOCITY_INJECTION, np.int32),
            origin=(1, c.ny - 2, 1), size=(c.nx - 2, 1, c.nz - 2))
    if c.amp:
        L.perturb((0, 0, 0), (c.nx, c.ny, c.nz), c.seed, c.amp)
    L.run(0, c.steps)
    return L


def mix(api):
    C = api.Cavity.make
    return [C((20, 18, 16), api.F32, 0.56, 0.17, 0.08, 17, 11, 1e-2),
            C((33, 15, 12), api.F16, 0.53, 0.17, 0.05, 24, 12, 2e-2),
            C((24, 20, 10), api.BF16, 0.6, 0.0, 0.1, 9, 13, 1e-2),
            C((18, 21, 19), api.F64, 0.55, 0.17, 0.07, 13, 14, 1e-2),
            C((64, 16, 12), api.F32, 0.52, 0.17, 0.1, 30, 15, 1e-2),
            C((12, 12, 12), api.F32, 0.7, 0.0, 0.02, 0, 16, 0.0),
            C((26, 14, 22), api.F16, 0.51, 0.17, 0.09, 21, 17, 0.0),
            C((40, 24, 14), api.F32, 0.55, 0.17, 0.06, 25, 18, 1e-2),
            C((10, 30, 12), api.F32, 0.58, 0.17, 0.05, 11, 19, 1e-2),
            # rows of whole 16-byte units: with shape 3 their beta steps are staged too
            C((32, 12, 14), api.F16, 0.54, 0.17, 0.06, 19, 20, 1e-2),
            C((16, 20, 18), api.F16, 0.57, 0.17, 0.04, 15, 21, 1e-2),
            C((32, 14, 12), api.C16, 0.55, 0.17, 0.07, 16, 22, 1e-2),
            C((21, 16, 13), api.C16, 0.6, 0.17, 0.05, 12, 23, 1e-2)]


@pytest.mark.parametrize("shape,use_graph", [(1, True), (2, True), (1, False), (3, True), (3, False)])
def test_batch_matches_lone_cavities(capi, shape, use_graph):
    api = capi
    cav = mix(api)
    B = api.Batch(cav, store_velocity=True)
    B.set_kernel_shape(shape)
    B.reset()
    B.run(use_graph=use_graph)
    assert B.status() == (0, 0)
    for c, L in zip(cav, B.lattices):
        R = lone(api, c)
        assert n_diff(L.read(api.FIELD_DD), R.read(api.FIELD_DD)) == 0
        if c.steps:
            assert n_diff(L.read(api.FIELD_VELOCITY), R.read(api.FIELD_VELOCITY)) == 0


def test_batch_autotuner_keeps_results(capi):
    api = capi
    cav = mix(api)
    B = api.Batch(cav, store_velocity=True)
    shape, ms = B.tune(trial_steps=6)
    assert shape in (1, 2, 3) and ms > 0
    B.run()
    for c, L in zip(cav, B.lattices):
        assert n_diff(L.read(api.FIELD_DD), lone(api, c).read(api.FIELD_DD)) == 0


def test_batch_partial_runs_add_up(capi):
    api = capi
    cav = mix(api)
    A = api.Batch(cav)
    A.reset()
    A.run()
    B = api.Batch(cav)
    B.reset()
    for _ in range(7):
        B.run(max_steps=5)
    B.run()
    for La, Lb in zip(A.lattices, B.lattices):
        assert n_diff(La.read(api.FIELD_DD), Lb.read(api.FIELD_DD)) == 0


@pytest.mark.parametrize("shape", [1, 3])
def test_server_results_do_not_depend_on_the_mix(capi, shape):
    """Solves admitted at different ticks, sharing launches with different
    neighbours, finish with the fields they have when run alone (shape 3:
    launches whose 16-bit members are all at an alpha step run the staged
    tiles, the others the one-cell kernel)."""
    api = capi
    cav = mix(api)
    S = api.Server(hbm_budget_bytes=64 << 20)
    S.set_kernel_shape(shape)
    ids = []
    finished = {}
    for k, c in enumerate(cav):
        ids.append(S.submit(c))
        S.tick(max_steps=3 + k)  # staggered admission, ragged ticks
        for sid in S.poll():
            finished[sid] = S.lattice(sid).read(api.FIELD_DD)
            S.release(sid)
    for _ in range(1000):
        if len(finished) == len(cav):
            break
        S.tick()
        for sid in S.poll():
            finished[sid] = S.lattice(sid).read(api.FIELD_DD)
            S.release(sid)
    assert S.status()["hbm_used"] == 0
    for sid, c in zip(ids, cav):
        assert n_diff(finished[sid], lone(api, c).read(api.FIELD_DD)) == 0


def test_server_admits_under_the_budget(capi):
    api = capi
    c = api.Cavity.make((32, 32, 32), api.F32, 0.6, 0.17, 0.05, 40)
    one = 32 ** 3 * 19 * 4 + 32 ** 3 + 32 ** 3 * 12 + 4096
    S = api.Server(hbm_budget_bytes=2.5 * one)
    a = [S.submit(c) for _ in range(4)]
    assert S.tick(max_steps=10) == 2  # two fit the budget, two wait
    st = S.status()
    assert st["active"] == 2 and st["queued"] == 2
    for _ in range(100):
        if S.poll():
            break
        S.tick()
    for sid in a[:2]:
        S.release(sid)
    assert S.tick(max_steps=1) == 2
    with pytest.raises(api.LbmError, match="does not fit"):
        S.submit(api.Cavity.make((128, 128, 128), api.F32, 0.6, 0.0, 0.05, 10))
