"""Parity of the CUDA path (through the C ABI) with the oracle and the reference.

Bar: bit-identical results.  The project's parity tolerances (per-step population
max-relative error 1e-6 in f32 and 1e-12 in f64) are asserted as well where a
test compares floating-point fields, but the kernels are built to reproduce
the reference arithmetic exactly and the tests demand equality of bits.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import golden_hashes, golden_small, max_rel, n_diff, state_hash

pytestmark = pytest.mark.gpu

SEED = 1234
TOL = {"f32": 1e-6, "f64": 1e-12, "f16": 1e-6, "bf16": 1e-6, "c16": 1e-6}


def gpu_params(api, p):
    return api.Params.make(p.inv_tau, p.tau0, p.les_c, p.gravity, p.lid, p.gravity_mode)


def gpu_single(api, O, dims, storage, p, lid=True, perturb=None, bc=None):
    L = api.Lattice(*dims, api.STORAGE_NAMES[storage], True, True)
    L.set_params(gpu_params(api, p))
    L.init(bc or [api.FLAG_OBSTACLE] * 6)
    if lid:
        nx, ny, nz = dims
        L.write(api.FIELD_FLAGS, np.full((nz - 2) * (nx - 2), api.FLAG_VELOCITY_INJECTION, np.int32),
                origin=(1, ny - 2, 1), size=(nx - 2, 1, nz - 2))
    if perturb is not None:
        L.perturb((0, 0, 0), dims, *perturb)
    return L


def snapshot(api, L):
    return (L.read(api.FIELD_DD), L.read(api.FIELD_VELOCITY), L.read(api.FIELD_DENSITY)[0],
            L.read(api.FIELD_FLAGS)[0])


def compare(api, O, L, sol, storage, where=""):
    dd, vel, rho, flags = snapshot(api, L)
    want = sol.k.decode(sol.lat.dd)
    assert n_diff(flags, sol.lat.flags) == 0, f"flags {where}"
    assert n_diff(dd, want) == 0, f"populations {where}: max rel {max_rel(dd, want):.3g}"
    assert max_rel(dd, want) <= TOL[storage]
    assert n_diff(vel, sol.lat.vel) == 0, f"velocity {where}"
    assert n_diff(rho, sol.lat.rho) == 0, f"density {where}"


def oracle_params(O, storage, dims, cs=0.0, gravity=(0.0, 0.0, 0.0), re=300.0, u=0.05, gravity_mode=0):
    rdt = O.STORAGE[storage][1]
    return O.Params.lattice(O.cavity_tau(u, dims[0], re), u, cs, dtype=rdt,
                            gravity=tuple(float(rdt(g)) for g in gravity), gravity_mode=gravity_mode)


@pytest.mark.parametrize("storage", ["f32", "f64", "f16", "bf16", "c16"])
def test_init_matches_oracle(capi, oracle_mod, storage):
    api, O = capi, oracle_mod
    dims = (13, 11, 9)
    bc = [1, 8, 1, 1, 8, 1]
    p = oracle_params(O, storage, dims)
    L = gpu_single(api, O, dims, storage, p, lid=False, bc=bc)
    s = O.Solver(O.OracleKernels(storage), dims, bc, p, storage)
    compare(api, O, L, s, storage, "after init")


@pytest.mark.parametrize("storage", ["f32", "f64", "f16", "bf16", "c16"])
@pytest.mark.parametrize("cs", [0.0, 0.17])
@pytest.mark.parametrize("gravity,gmode", [((0.0, 0.0, 0.0), 0), ((1e-5, -2e-5, 3e-6), 0),
                                           ((1e-5, -2e-5, 3e-6), 1)])
@pytest.mark.parametrize("dims,shape", [((21, 14, 11), 1), ((22, 14, 11), 2), ((64, 12, 18), 2),
                                        ((21, 14, 11), 3), ((64, 12, 18), 3)])
def test_steps_match_oracle(capi, oracle_mod, storage, cs, gravity, gmode, dims, shape):
    """Perturbed lid cavity: every array, every step, for the one-cell, the
    two-cell (needs an even x extent; the 64-wide case has whole warps inside
    the lattice) and the staged-tile kernel shapes (the 64x12x18 case spans
    many tiles and ends in a partial one), with the reference's gravity terms
    and with the optional per-term forcing."""
    api, O = capi, oracle_mod
    p = oracle_params(O, storage, dims, cs, gravity, gravity_mode=gmode)
    L = gpu_single(api, O, dims, storage, p, perturb=(SEED, 2e-2))
    L.set_kernel_shape(shape)
    s = O.single(O.OracleKernels(storage), dims, p, storage)
    s.k.perturb(s.lat, (0, 0, 0), dims, SEED, 2e-2)
    compare(api, O, L, s, storage, "after start-up")
    for k in range(12):
        L.step(s.lat.counter & 1)
        s.step()
        compare(api, O, L, s, storage, f"after step {k + 1}")


@pytest.mark.parametrize("storage,shape", [("f32", 1), ("f16", 3)])
def test_parity_detects_a_planted_mistake(capi, oracle_mod, storage, shape):
    """Negative control: with the oracle's BGK relaxation rate moved (the
    mistake planted on the CPU side) -- by one unit in the last place for
    float, by 2^-7 relative for half storage, whose 11-bit populations absorb
    smaller changes -- the CUDA populations no longer match it."""
    import dataclasses

    api, O = capi, oracle_mod
    dims = (64, 12, 18)
    p = oracle_params(O, storage, dims)
    L = gpu_single(api, O, dims, storage, p, perturb=(SEED, 2e-2))
    L.set_kernel_shape(shape)
    inv = np.float32(p.inv_tau)
    inv = np.nextafter(inv, np.float32(2)) if storage == "f32" else np.float32(inv * (1 + 2.0 ** -7))
    s = O.single(O.OracleKernels(storage), dims, dataclasses.replace(p, inv_tau=float(inv)), storage)
    s.k.perturb(s.lat, (0, 0, 0), dims, SEED, 2e-2)
    differs = 0
    for _ in range(4):
        L.step(s.lat.counter & 1)
        s.step()
        differs += n_diff(L.read(api.FIELD_DD), s.k.decode(s.lat.dd))
    assert differs > 0


@pytest.mark.parametrize("storage", ["f32", "f64"])
def test_matches_reference_arrays(capi, oracle_mod, storage):
    """Full arrays written by the reference kernels (tests/golden)."""
    api, O = capi, oracle_mod
    g = golden_small(storage)
    dims = (12, 8, 8)
    rdt = O.STORAGE[storage][1]
    p = O.Params.lattice(O.cavity_tau(0.05, 12, 100.0), 0.05, dtype=rdt,
                         gravity=tuple(float(rdt(x)) for x in (1e-5, -2e-5, 3e-6)))
    L = gpu_single(api, O, dims, storage, p, perturb=(SEED, 1e-2))
    assert n_diff(L.read(api.FIELD_DD), g["dd0"]) == 0
    for k in range(1, 9):
        L.step((k - 1) & 1)
        if f"dd{k}" in g:
            dd, vel, rho, flags = snapshot(api, L)
            assert n_diff(dd, g[f"dd{k}"]) == 0, f"step {k}"
            assert n_diff(vel, g[f"vel{k}"]) == 0, f"step {k}"
            assert n_diff(rho, g[f"rho{k}"]) == 0, f"step {k}"


@pytest.mark.parametrize("storage,shape", [("f32", 1), ("f32", 2), ("f32", 3), ("f64", 1)])
def test_c1_matches_reference_every_step(capi, oracle_mod, storage, shape):
    """Config 1 geometry (64^3 lid cavity, Re 1000, U 0.05, rest start) with
    the reference's plain BGK: the state hash equals the reference kernels'
    after every step (100 steps f32, 40 f64)."""
    api, O = capi, oracle_mod
    ref = golden_hashes()[f"c1_{storage}"]
    dims = (64, 64, 64)
    rdt = O.STORAGE[storage][1]
    p = O.Params.lattice(O.cavity_tau(0.05, 64, 1000.0), 0.05, dtype=rdt)
    L = gpu_single(api, O, dims, storage, p)
    L.set_kernel_shape(shape)
    flags = L.read(api.FIELD_FLAGS)[0]
    m = O.fluid_mask(flags)

    def h():
        dd, vel, rho, fl = snapshot(api, L)
        return state_hash(dd, vel, rho, fl, m)

    assert h() == ref[0]
    for k in range(1, len(ref)):
        L.step((k - 1) & 1)
        assert h() == ref[k], f"step {k}"


def test_c1_smagorinsky_matches_oracle(capi, oracle_mod):
    """Config 1 as specified: 64^3, Re 1000, U 0.05, Cs 0.17, f32, 100 steps,
    populations, density and velocity compared every step."""
    api, O = capi, oracle_mod
    dims = (64, 64, 64)
    p = O.Params.lattice(O.cavity_tau(0.05, 64, 1000.0), 0.05, 0.17, dtype=np.float32)
    L = gpu_single(api, O, dims, "f32", p)
    s = O.single(O.OracleKernels("f32"), dims, p, "f32")
    for k in range(100):
        L.step(k & 1)
        s.step()
        compare(api, O, L, s, "f32", f"after step {k + 1}")


@pytest.mark.parametrize("use_graph,shape", [(False, 1), (True, 1), (True, 2), (True, 3), (False, 3)])
def test_domain_matches_reference_decomposition(capi, oracle_mod, use_graph, shape):
    """2x2x1 decomposition on one GPU: every subdomain's state hash equals the
    reference kernels' with the reference host exchange, every step."""
    api, O = capi, oracle_mod
    ref = golden_hashes()["decomposed_f32"]
    p = O.Params.lattice(O.cavity_tau(0.1, 22, 1000.0), 0.1, dtype=np.float32)
    D = api.Domain((24, 16, 16), (2, 2, 1), api.F32, True, True)
    D.set_params(gpu_params(api, p))
    D.set_kernel_shape(shape)
    D.reset()
    D.perturb(SEED, 1e-2)
    done = 0
    while done < len(ref):
        n = min(2, len(ref) - done) if use_graph else 1
        D.run(n, use_graph)  # pairs of steps replay the captured graph
        done += n
        assert D.counter == done
        got = []
        for L in D.subdomains:
            dd, vel, rho, fl = snapshot(api, L)
            got.append(state_hash(dd, vel, rho, fl, O.fluid_mask(fl)))
        assert got == ref[done - 1], f"step {done}"


@pytest.mark.parametrize("storage,size,nums,halo_mode", [
    ("f32", (30, 20, 12), (2, 2, 1), 0), ("f64", (30, 20, 12), (2, 2, 1), 0),
    ("f16", (30, 20, 12), (2, 2, 1), 0), ("f32", (36, 24, 24), (3, 2, 2), 1),
    ("bf16", (36, 24, 24), (2, 1, 3), 1),
    # subdomains 32 and 16 cells wide: the staged beta tiles (two cells per
    # thread with the subgrid model) run over ghost layers
    ("f16", (64, 24, 20), (2, 2, 1), 1), ("bf16", (48, 16, 24), (3, 1, 2), 0),
    # 64 subdomains: 96 copies per exchange phase, more than one launch's
    # parameter space holds
    ("f32", (24, 24, 24), (4, 4, 4), 0), ("f16", (24, 24, 24), (4, 4, 4), 1),
    # the 16-bit float of this project, staged beta tiles over ghost layers
    ("c16", (64, 24, 20), (2, 2, 1), 1), ("c16", (30, 20, 12), (2, 2, 1), 0)])
def test_domain_matches_oracle_with_subgrid_model(capi, oracle_mod, storage, size, nums, halo_mode):
    api, O = capi, oracle_mod
    p = oracle_params(O, storage, (28, 0, 0), cs=0.17, re=5000.0, u=0.1)
    D = api.Domain(size, nums, api.STORAGE_NAMES[storage], True, True)
    D.set_params(gpu_params(api, p))
    D.set_halo_mode(halo_mode)
    D.reset()
    D.perturb(SEED, 1e-2)
    R = O.Domain(lambda d: O.OracleKernels(storage), size, nums, p, storage, halo_mode=halo_mode)
    R.perturb(SEED, 1e-2)
    for _ in range(3):
        D.run(5, True)
        for _ in range(5):
            R.step()
        for L, (_, s, _) in zip(D.subdomains, R.parts):
            compare(api, O, L, s, storage, f"after step {R.counter}")


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_domain_view_over_own_lattices(capi, storage):
    """lbm_cu_domain_wrap over lattices initialised elsewhere steps them
    exactly as the owning domain does (graph replay, odd start counters, and
    parameters changed through the lattices' own handles)."""
    api = capi
    size, nums = (48, 32, 16), (2, 2, 1)
    st = api.STORAGE_NAMES[storage]

    def made():
        D = api.Domain(size, nums, st, True, True)
        D.set_params(api.Params.make(1.0 / 0.56, 0.56, api.les_coefficient(0.17), (0, 0, 0), 0.08))
        D.reset()
        D.perturb(SEED, 1e-2)
        return D

    A, B = made(), made()
    V = api.Domain.wrap(B.subdomains, size, nums)
    A.run(7, True)
    V.counter = 0
    V.run(7, True)
    assert V.counter == 7
    p2 = api.Params.make(1.0 / 0.61, 0.61, api.les_coefficient(0.1), (0, 0, 0), 0.05)
    A.set_params(p2)
    for L in B.subdomains:
        L.set_params(p2)
    A.run(6, True)
    V.run(6, True)
    for La, Lb in zip(A.subdomains, B.subdomains):
        for f in (api.FIELD_DD, api.FIELD_VELOCITY, api.FIELD_DENSITY):
            assert n_diff(La.read(f), Lb.read(f)) == 0
    V.close()
    assert n_diff(B.subdomains[0].read(api.FIELD_DD), A.subdomains[0].read(api.FIELD_DD)) == 0  # lattices kept


def test_domain_equals_single_domain(capi, oracle_mod):
    """Validate mode on the GPU: decomposed interior velocity equals the
    reduced single domain bit for bit (src/main.cpp:309-408)."""
    api, O = capi, oracle_mod
    size, nums = (40, 32, 16), (2, 2, 1)
    red = tuple(s - 2 * (n - 1) for s, n in zip(size, nums))
    p = oracle_params(O, "f32", (red[0], 0, 0), cs=0.17, re=2000.0, u=0.1)
    D = api.Domain(size, nums, api.F32, True, True)
    D.set_params(gpu_params(api, p))
    D.reset()
    D.perturb(SEED, 1e-2)
    S = gpu_single(api, O, red, "f32", p, perturb=(SEED, 1e-2))
    D.run(40, True)
    for k in range(40):
        S.step(k & 1)
    vs = S.read(api.FIELD_VELOCITY)
    sx, sy, sz = D.sub
    for i, L in enumerate(D.subdomains):
        c = (i % 2, (i // 2) % 2, 0)
        o = tuple(ci * (si - 2) for ci, si in zip(c, D.sub))
        loc = L.read(api.FIELD_VELOCITY)[:, 1:sz - 1, 1:sy - 1, 1:sx - 1]
        glob = vs[:, o[2] + 1:o[2] + sz - 1, o[1] + 1:o[1] + sy - 1, o[0] + 1:o[0] + sx - 1]
        assert n_diff(loc, glob) == 0


def test_rect_io_and_masked_write(capi):
    api = capi
    L = api.Lattice(10, 9, 8, api.F32, True, True)
    L.init([1] * 6)
    rng = np.random.default_rng(1)
    o, sz = (2, 1, 3), (5, 4, 2)
    src = rng.random((19, 2, 4, 5), dtype=np.float32)
    L.write(api.FIELD_DD, src, o, sz)
    assert n_diff(L.read(api.FIELD_DD, o, sz), src) == 0
    before = L.read(api.FIELD_DD)
    src2 = rng.random((19, 2, 4, 5), dtype=np.float32)
    L.write(api.FIELD_DD, src2, o, sz, norm=(0, 0, -1))  # planes with e_z < 0
    after = L.read(api.FIELD_DD)
    sel = [f for f in range(19) if -O_E(f)[2] > 0]
    for f in range(19):
        region = after[f, 3:5, 1:5, 2:7]
        assert n_diff(region, src2[f] if f in sel else before[f, 3:5, 1:5, 2:7]) == 0
    v = rng.random((3, 8, 9, 10), dtype=np.float32)
    L.write(api.FIELD_VELOCITY, v)
    assert n_diff(L.read(api.FIELD_VELOCITY), v) == 0
    fl = rng.integers(0, 16, (1, 8, 9, 10)).astype(np.int32)
    L.write(api.FIELD_FLAGS, fl)
    assert n_diff(L.read(api.FIELD_FLAGS), fl) == 0
    with pytest.raises(api.LbmError, match="flag values"):
        L.write(api.FIELD_FLAGS, np.full((1, 1, 1, 1), 300, np.int32), (0, 0, 0), (1, 1, 1))
    with pytest.raises(api.LbmError, match="outside"):
        L.read(api.FIELD_DD, (8, 0, 0), (5, 1, 1))


def O_E(f):
    from oracle.oracle import E

    return E[f]


def test_halo_copies_selected_planes(capi):
    api = capi
    a = api.Lattice(8, 7, 6, api.F64, False, False)
    b = api.Lattice(8, 7, 6, api.F64, False, False)
    rng = np.random.default_rng(2)
    da = rng.random((19, 6, 7, 8))
    db = rng.random((19, 6, 7, 8))
    a.write(api.FIELD_DD, da)
    b.write(api.FIELD_DD, db)
    api.halo(a, (6, 0, 0), b, (0, 0, 0), (1, 7, 6), norm=(1, 0, 0))
    got = b.read(api.FIELD_DD)
    for f in range(19):
        want = da[f, :, :, 6] if O_E(f)[0] > 0 else db[f, :, :, 0]
        assert n_diff(got[f, :, :, 0], want) == 0
        assert n_diff(got[f, :, :, 1:], db[f, :, :, 1:]) == 0


@pytest.mark.parametrize("storage", ["f32", "f64", "f16", "c16"])
def test_reduce_conserved(capi, oracle_mod, storage):
    api, O = capi, oracle_mod
    dims = (24, 20, 18)
    p = oracle_params(O, storage, dims, cs=0.17)
    L = gpu_single(api, O, dims, storage, p, perturb=(SEED, 3e-2))
    for k in range(7):
        L.step(k & 1)
    dd = L.read(api.FIELD_DD).astype(np.float64)
    fl = L.read(api.FIELD_FLAGS)[0]
    m = fl == api.FLAG_FLUID
    layout = 0  # the 7th step (counter 6) is a beta step: standard slots
    f = dd[:, m]
    if layout:
        f = f[O.OPP]
    E = O.E.astype(np.float64)
    rho = f.sum(0)
    j = E.T @ f
    want = np.array([rho.sum(), j[0].sum(), j[1].sum(), j[2].sum(), 0.5 * (j ** 2).sum()])
    got = L.reduce_conserved(layout)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-13)


def test_errors_are_reported(capi):
    api = capi
    with pytest.raises(api.LbmError, match="at least 3"):
        api.Lattice(2, 5, 5)
    with pytest.raises(api.LbmError, match="does not match"):
        api.Domain((30, 20, 10), (4, 1, 1))
    L = api.Lattice(5, 5, 5, api.F32, False, False)
    with pytest.raises(api.LbmError, match="velocity is not stored"):
        L.read(api.FIELD_VELOCITY)


@pytest.mark.parametrize("size,nums,halo_mode", [((30, 20, 12), (2, 2, 1), 0), ((36, 24, 24), (3, 2, 2), 1),
                                                 ((6, 8, 8), (2, 1, 1), 0), ((24, 24, 24), (4, 4, 4), 1),
                                                 ((256, 64, 32), (2, 2, 1), 1)])
def test_fused_x_exchange_equals_separate_launch(capi, size, nums, halo_mode):
    """The x part of the exchange after alpha done by the one-cell alpha
    kernel itself gives the same bits as its own copy launch: subdomains of
    three cells in x (the x = 1 cells send both ways), 64 subdomains, the
    benchmark's subdomain width; runs ending on a beta and on an alpha step."""
    api = capi

    def run(fused):
        D = api.Domain(size, nums, api.F32, True, True)
        D.set_params(api.Params.make(1.0 / 0.52, 0.52, api.les_coefficient(0.17), (0, 0, 0), 0.09))
        D.set_halo_mode(halo_mode)
        D.set_fused_exchange(fused)
        D.reset()
        D.perturb(SEED, 1e-2)
        D.run(5, use_graph=False)
        out = [[L.read(api.FIELD_DD) for L in D.subdomains]]
        D.set_store_interval(0)
        for steps in (8, 3):
            D.run(steps, use_graph=True)
            out.append([L.read(f) for L in D.subdomains for f in (api.FIELD_DD, api.FIELD_VELOCITY, api.FIELD_DENSITY)])
        return out

    for a, b in zip(run(True), run(False)):
        for x, y in zip(a, b):
            assert n_diff(x, y) == 0


@pytest.mark.parametrize("nums", [(2, 1, 1), (2, 2, 2)])
def test_fused_exchange_with_obstacles_at_the_interface(capi, nums):
    """Obstacle cells next to an x interface, whose alpha steps leave their
    populations alone but still send the x faces to the neighbour's ghost
    layer: the alpha kernel's copies give the bits of the copy launches;
    runs ending on an alpha and on a beta step."""
    api = capi
    size = (24, 16, 12)
    sub = [s // n for s, n in zip(size, nums)]

    def run(fused):
        D = api.Domain(size, nums, api.F32, True, True)
        D.set_params(api.Params.make(1.0 / 0.53, 0.53, api.les_coefficient(0.17), (0, 0, 0), 0.08))
        D.set_fused_exchange(fused)
        D.reset()
        D.perturb(SEED, 1e-2)
        box = (2, min(4, sub[1] - 3), min(3, sub[2] - 2))
        for i, L in enumerate(D.subdomains):
            x0 = 1 if (i % nums[0]) else sub[0] - 3  # next to the interface on both sides
            L.write(api.FIELD_FLAGS, np.full(box[0] * box[1] * box[2], api.FLAG_OBSTACLE, np.int32),
                    origin=(x0, 1, 1), size=box)
        out = []
        for steps, graph in ((4, False), (7, False), (6, True), (5, True)):
            D.run(steps, use_graph=graph)
            out.append([[L.read(f) for f in (api.FIELD_DD, api.FIELD_VELOCITY, api.FIELD_DENSITY)]
                        for L in D.subdomains])
        return out

    for a, b in zip(run(True), run(False)):
        for sa, sb in zip(a, b):
            for x, y in zip(sa, sb):
                assert n_diff(x, y) == 0


@pytest.mark.parametrize("storage", ["f16", "bf16", "c16"])
def test_deviation_stats_match_the_stored_bits(capi, oracle_mod, storage):
    """lbm_cu_deviation_stats against the oracle's stored bits (the two are
    bit-identical): counts of zero, subnormal and saturated deviations over
    the fluid cells, and the largest magnitude."""
    api, O = capi, oracle_mod
    dims = (32, 20, 16)
    p = oracle_params(O, storage, dims, cs=0.17, u=0.1)
    L = gpu_single(api, O, dims, storage, p, perturb=(SEED, 3e-2))
    s = O.single(O.OracleKernels(storage), dims, p, storage)
    s.k.perturb(s.lat, (0, 0, 0), dims, SEED, 3e-2)
    for _ in range(5):
        L.step(s.lat.counter & 1)
        s.step()
    got = api.deviation_stats(L)
    raw = s.lat.dd[:, s.lat.flags == O.FLAG_FLUID]
    b = raw.view(np.uint16).astype(np.int64)
    ebits, mbits = {"f16": (5, 10), "bf16": (8, 7), "c16": (3, 12)}[storage]
    e, m = (b >> mbits) & ((1 << ebits) - 1), b & ((1 << mbits) - 1)
    top = (1 << ebits) - 1
    sat = (b & 0x7fff) == (0x7fff if storage == "c16" else ((top << mbits) - 1))
    if storage != "c16":
        sat |= e == top
    assert got["values"] == b.size
    assert got["zero"] == int(((e == 0) & (m == 0)).sum())
    assert got["subnormal"] == int(((e == 0) & (m != 0)).sum())
    assert got["saturated"] == int(sat.sum())
    if storage == "f16":
        dev = raw.astype(np.float64)
    elif storage == "bf16":
        dev = (raw.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    else:
        from test_oracle_pin import _c16_value
        dev = _c16_value(raw)
    assert got["max_abs"] == np.abs(dev).max()


@pytest.mark.parametrize("storage,steps,every", [("f32", 7, 1), ("f16", 6, 1), ("f32", 9, 4)])
def test_timed_graph_run_equals_eager_steps(capi, storage, steps, every):
    """lbm_cu_domain_prepare_timed_run: the captured run with an event pair
    around every step kernel gives the bits of step-by-step launches and
    times exactly `steps` kernels, split into beta and alpha steps; a run of
    another length does not use it."""
    api = capi
    size, nums = (48, 32, 16), (2, 2, 1)

    def made():
        D = api.Domain(size, nums, api.STORAGE_NAMES[storage], True, True)
        D.set_params(api.Params.make(1.0 / 0.56, 0.56, api.les_coefficient(0.17), (0, 0, 0), 0.08))
        D.set_store_interval(0)
        D.reset()
        D.perturb(SEED, 1e-2)
        D.run(3, use_graph=False)
        return D

    A, B = made(), made()
    A.run(steps, use_graph=False)
    B.profile(True)
    B.kernel_time(reset=True)
    B.prepare_timed_run(steps, every)
    B.run(steps, use_graph=True)
    (b_ms, b_n), (a_ms, a_n) = B.kernel_time_by_step()
    ms, n = B.kernel_time(reset=True)
    assert n == sum(1 for k in range(steps) if k % every < 2) and ms > 0
    # step k runs on counter 3 + k: beta on an even counter, alpha on an odd one
    assert b_n == sum(1 for k in range(steps) if k % every < 2 and (3 + k) % 2 == 0)
    assert a_n == n - b_n and b_ms > 0 and a_ms > 0
    assert abs(b_ms + a_ms - ms) <= 1e-9 * max(1.0, ms)
    assert B.counter == A.counter == 3 + steps
    for La, Lb in zip(A.subdomains, B.subdomains):
        for f in (api.FIELD_DD, api.FIELD_VELOCITY, api.FIELD_DENSITY):
            assert n_diff(La.read(f), Lb.read(f)) == 0
    B.run(steps + 1, use_graph=True)  # another length: the ordinary path (step by step while profiling)
    ms2, n2 = B.kernel_time(reset=True)
    assert n2 == steps + 1
