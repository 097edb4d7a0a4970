"""The conservation sums through the no-allocation entry point.

lbm_cu_reduce_conserved_noalloc serves callers that must not allocate device
memory (a serving loop whose HBM is all handed out under a budget, a monitor
that must not trigger cudaMalloc's implicit synchronisation).  It keeps its
partial sums in a fixed array inside the library instead of a staging
buffer, so its results must equal those of lbm_cu_reduce_conserved -- on two
calls in a row, because the array keeps the previous call's contents.
This file is collected last so that a failure here cannot hide the others.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 1234


def _lattice(api, O, dims, storage, steps):
    rdt = O.STORAGE[storage][1]
    p = O.Params.lattice(O.cavity_tau(0.05, dims[0], 500.0), 0.05, 0.17, dtype=rdt)
    L = api.Lattice(*dims, api.STORAGE_NAMES[storage], False, False)
    L.set_params(api.Params.make(p.inv_tau, p.tau0, p.les_c, p.gravity, p.lid))
    L.init([api.FLAG_OBSTACLE] * 6)
    L.perturb((0, 0, 0), dims, SEED, 3e-2)
    for k in range(steps):
        L.step(k & 1)
    return L


@pytest.mark.parametrize("storage,dims,steps", [("f32", (48, 40, 36), 5), ("f64", (30, 26, 22), 4),
                                                ("f16", (64, 64, 40), 3), ("bf16", (64, 48, 40), 3),
                                                ("c16", (32, 40, 24), 3)])
def test_noalloc_sums_equal_allocating_sums(capi, oracle_mod, storage, dims, steps):
    api, O = capi, oracle_mod
    L = _lattice(api, O, dims, storage, steps)
    layout = (steps - 1) & 1  # last step beta -> standard slots (0), alpha -> opposite slots (1)
    for _ in range(2):  # the shared array keeps the previous call's partials
        want = L.reduce_conserved(layout)
        got = L.reduce_conserved_noalloc(layout)
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-13)


def test_noalloc_after_a_larger_lattice(capi, oracle_mod):
    """A small lattice after a large one reads only the partials it wrote."""
    api, O = capi, oracle_mod
    big = _lattice(api, O, (128, 96, 80), "f32", 2)
    small = _lattice(api, O, (20, 18, 16), "f32", 2)
    for L in (big, small, big):
        np.testing.assert_allclose(L.reduce_conserved_noalloc(1), L.reduce_conserved(1), rtol=1e-12, atol=1e-13)


def test_noalloc_rejects_lattices_beyond_its_limit(capi):
    api = capi
    L = api.Lattice(514, 512, 512, api.F16, False, False)  # 134,742,016 cells > 512^3
    with pytest.raises(api.LbmError, match="handles at most 134217728"):
        L.reduce_conserved_noalloc(0)


def test_noalloc_at_its_limit(capi):
    """A 512^3 lattice fills all 16384 partials of the array."""
    api = capi
    L = api.Lattice(512, 512, 512, api.F16, False, False)
    L.init([api.FLAG_OBSTACLE] * 6)
    L.perturb((0, 0, 0), (512, 512, 512), SEED, 3e-2)  # writes the opposite-slot layout
    for _ in range(2):
        np.testing.assert_allclose(L.reduce_conserved_noalloc(1), L.reduce_conserved(1), rtol=1e-12, atol=1e-13)
