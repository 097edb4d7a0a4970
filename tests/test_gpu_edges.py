"""Edge sizes: the smallest lattices against the oracle, and a lattice of
almost 2^31 cells (the largest the 32-bit cell indexing admits) whose kernel
shapes must agree bit for bit with each other."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import n_diff

pytestmark = pytest.mark.gpu

SEED = 4242


def params(api, storage, cs=0.17, tau=0.53):
    t = np.float64(tau) if storage == api.F64 else np.float32(tau)
    inv = float(1.0 / t) if storage == api.F64 else float(np.float32(1) / t)
    return api.Params.make(inv, float(t), api.les_coefficient(cs), (0.0, 0.0, 0.0), 0.07)


@pytest.mark.parametrize("storage", ["f32", "f64", "f16", "bf16", "c16"])
@pytest.mark.parametrize("dims", [(3, 3, 3), (4, 3, 5), (3, 7, 3), (9, 3, 4)])
@pytest.mark.parametrize("shape", [1, 2, 3])
def test_smallest_lattices_match_oracle(capi, oracle_mod, storage, dims, shape):
    """Lattices of 3 cells along an axis (walls only in that direction, every
    neighbour wraps) through every kernel shape, every step."""
    api, O = capi, oracle_mod
    rdt = O.STORAGE[storage][1]
    t = rdt(0.53)
    p = O.Params(inv_tau=float(rdt(1) / t), tau0=float(t), les_c=float(rdt(O.les_coefficient(0.17))),
                 lid=float(rdt(0.07)))
    L = api.Lattice(*dims, api.STORAGE_NAMES[storage], True, True)
    L.set_params(api.Params.make(p.inv_tau, p.tau0, p.les_c, p.gravity, p.lid))
    L.init([api.FLAG_OBSTACLE] * 6)
    nx, ny, nz = dims
    if nx > 2 and nz > 2:
        L.write(api.FIELD_FLAGS, np.full((nz - 2) * (nx - 2), api.FLAG_VELOCITY_INJECTION, np.int32),
                origin=(1, ny - 2, 1), size=(nx - 2, 1, nz - 2))
    L.perturb((0, 0, 0), dims, SEED, 2e-2)
    L.set_kernel_shape(shape)
    s = O.single(O.OracleKernels(storage), dims, p, storage)
    s.k.perturb(s.lat, (0, 0, 0), dims, SEED, 2e-2)
    for k in range(6):
        L.step(s.lat.counter & 1)
        s.step()
        assert n_diff(L.read(api.FIELD_DD), s.k.decode(s.lat.dd)) == 0, f"step {k + 1}"


def test_lattice_of_almost_2_31_cells(capi):
    """1290^3 = 2,146,689,000 cells of shifted half storage (82 GB): the
    one-cell and the staged kernels give identical populations and identical
    FP64 conservation sums after a beta and an alpha step; one cell more per
    axis exceeds the 32-bit cell range and is refused."""
    api = capi
    dims = (1290, 1290, 1290)
    with pytest.raises(api.LbmError, match="2\\^31"):
        api.Lattice(1291, 1291, 1291, api.F16, False, False)
    L = api.Lattice(*dims, api.F16, False, False)
    L.set_params(params(api, api.F16))
    boxes = [((0, 0, 0), (8, 8, 8)), ((1282, 1282, 1282), (8, 8, 8)), ((641, 1283, 600), (16, 7, 9))]
    res = []
    for shape in (1, 3):
        L.init([api.FLAG_OBSTACLE] * 6)
        L.write(api.FIELD_FLAGS, np.full(4, api.FLAG_VELOCITY_INJECTION, np.int32),
                origin=(640, 1288, 640), size=(2, 1, 2))
        L.perturb((0, 0, 0), dims, SEED, 1e-3)
        L.set_kernel_shape(shape)
        L.run(0, 2)
        res.append(([L.read(api.FIELD_DD, origin=o, size=z) for o, z in boxes], L.reduce_conserved(1)))
    for a, b in zip(res[0][0], res[1][0]):
        assert n_diff(a, b) == 0
    assert np.array_equal(res[0][1], res[1][1])
    # the start-up field holds rho = 1: the mass sum over the fluid cells is their count
    assert abs(res[0][1][0] / (1288 ** 3 - 4) - 1.0) < 1e-4
