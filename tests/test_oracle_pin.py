"""The C oracle, pinned against the reference's own kernels (CPU only).

The reference pins nothing itself: it ships no tests and no golden vectors.
The pins are the reference's kernel source run on the same inputs -- live
through oracle/build_ref.py where the reference tree is present, otherwise
through the fixtures tests/golden/make_golden.py wrote from it.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import bits, golden_hashes, golden_small, n_diff, state_hash

SEED = 1234


def _small_params(O, storage):
    rdt = O.STORAGE[storage][1]
    return O.Params.lattice(O.cavity_tau(0.05, 12, 100.0), 0.05, dtype=rdt,
                            gravity=tuple(float(rdt(g)) for g in (1e-5, -2e-5, 3e-6)))


@pytest.mark.parametrize("storage", ["f32", "f64"])
def test_oracle_reproduces_reference_arrays(oracle_mod, storage):
    """Full arrays of a perturbed lid cavity with gravity, 8 steps (both parities)."""
    O = oracle_mod
    g = golden_small(storage)
    dims = (12, 8, 8)
    s = O.single(O.OracleKernels(storage), dims, _small_params(O, storage), storage)
    s.k.perturb(s.lat, (0, 0, 0), dims, SEED, 1e-2)
    assert n_diff(s.lat.dd, g["dd0"]) == 0
    assert n_diff(s.lat.flags, g["flags"]) == 0
    for k in range(1, 9):
        s.step()
        if f"dd{k}" in g:
            assert n_diff(s.lat.dd, g[f"dd{k}"]) == 0, f"populations differ after step {k}"
            assert n_diff(s.lat.vel, g[f"vel{k}"]) == 0, f"velocity differs after step {k}"
            assert n_diff(s.lat.rho, g[f"rho{k}"]) == 0, f"density differs after step {k}"


@pytest.mark.parametrize("storage,wg", [("f32", 128), ("f32", 0), ("f64", 128)])
def test_oracle_reproduces_reference_c1_hashes(oracle_mod, storage, wg):
    """64^3 lid cavity, Re 1000, U 0.05: every step's fluid and lid state equals
    the reference's.  wg=128 reproduces the reference beta kernel's work-group
    realignment (64 divides 128); wg=0 is the plain linear wrap the CUDA
    kernels use -- the masked state is the same either way."""
    O = oracle_mod
    ref = golden_hashes()[f"c1_{storage}"]
    rdt = O.STORAGE[storage][1]
    p = O.Params.lattice(O.cavity_tau(0.05, 64, 1000.0), 0.05, dtype=rdt, wg=wg)
    s = O.single(O.OracleKernels(storage), (64, 64, 64), p, storage)
    m = O.fluid_mask(s.lat.flags)
    assert state_hash(s.lat.dd, s.lat.vel, s.lat.rho, s.lat.flags, m) == ref[0]
    for k in range(1, len(ref)):
        s.step()
        assert state_hash(s.lat.dd, s.lat.vel, s.lat.rho, s.lat.flags, m) == ref[k], f"step {k}"


@pytest.mark.parametrize("plant", ["inv_tau", "lid"])
def test_pin_detects_a_one_ulp_mistake(oracle_mod, plant):
    """Negative control of the pin above: the oracle with one parameter moved
    by one unit in the last place (a mistake planted on the CPU) leaves the
    reference's hashes within a few steps."""
    O = oracle_mod
    ref = golden_hashes()["c1_f32"]
    p = O.Params.lattice(O.cavity_tau(0.05, 64, 1000.0), 0.05, dtype=np.float32, wg=0)
    if plant == "inv_tau":
        p.inv_tau = float(np.nextafter(np.float32(p.inv_tau), np.float32(2)))
    else:
        p.lid = float(np.nextafter(np.float32(p.lid), np.float32(1)))
    s = O.single(O.OracleKernels("f32"), (64, 64, 64), p, "f32")
    m = O.fluid_mask(s.lat.flags)
    differs = False
    for k in range(1, min(len(ref), 6)):
        s.step()
        differs = differs or state_hash(s.lat.dd, s.lat.vel, s.lat.rho, s.lat.flags, m) != ref[k]
    assert differs


def test_oracle_reproduces_reference_decomposed_hashes(oracle_mod):
    O = oracle_mod
    ref = golden_hashes()["decomposed_f32"]
    p = O.Params.lattice(O.cavity_tau(0.1, 22, 1000.0), 0.1, dtype=np.float32)
    D = O.Domain(lambda d: O.OracleKernels("f32"), (24, 16, 16), (2, 2, 1), p, "f32")
    D.perturb(SEED, 1e-2)
    for k, want in enumerate(ref):
        D.step()
        got = [state_hash(s.lat.dd, s.lat.vel, s.lat.rho, s.lat.flags, O.fluid_mask(s.lat.flags))
               for _, s, _ in D.parts]
        assert got == want, f"step {k + 1}"


def _have_reference():
    from oracle import build_ref

    return build_ref.available()


@pytest.mark.skipif(not _have_reference(), reason="reference tree not present on this machine")
@pytest.mark.parametrize("storage,dims,wg", [("f32", (16, 8, 8), 64), ("f64", (16, 8, 8), 64),
                                             ("f32", (20, 16, 8), 128), ("f64", (12, 16, 8), 128)])
def test_oracle_equals_reference_live(oracle_mod, storage, dims, wg):
    """Bit equality of every array, every step, against the reference kernels
    compiled from the reference tree; gravity and a perturbed start on."""
    O = oracle_mod
    rdt = O.STORAGE[storage][1]
    mk = lambda w: O.Params.lattice(O.cavity_tau(0.05, dims[0], 300.0), 0.05, dtype=rdt, wg=w,
                                    gravity=tuple(float(rdt(g)) for g in (2e-5, -1e-5, 5e-6)))
    a = O.single(O.OracleKernels(storage), dims, mk(wg), storage)
    b = O.single(O.RefKernels(storage, *dims, wg), dims, mk(0), storage)
    for s in (a, b):
        O.OracleKernels(storage).perturb(s.lat, (0, 0, 0), dims, SEED, 2e-2)
    for k in range(30):
        a.step()
        b.step()
        for name in ("dd", "vel", "rho", "flags"):
            assert n_diff(getattr(a.lat, name), getattr(b.lat, name)) == 0, f"{name} step {k + 1}"


@pytest.mark.skipif(not _have_reference(), reason="reference tree not present on this machine")
def test_linear_wrap_differs_only_in_wall_slots(oracle_mod):
    """Where the reference beta kernel realigns x inside a work-group, the
    linear-wrap kernels differ from it only in wall-cell populations."""
    O = oracle_mod
    p0 = O.Params.lattice(O.cavity_tau(0.1, 30, 1000.0), 0.1, dtype=np.float32)
    A = O.Domain(lambda d: O.OracleKernels("f32"), (32, 24, 16), (2, 2, 1), p0, "f32")
    B = O.Domain(lambda d: O.RefKernels("f32", *d, 128), (32, 24, 16), (2, 2, 1), p0, "f32")
    for D in (A, B):
        D.perturb(SEED, 1e-2)
    for _ in range(20):
        A.step()
        B.step()
        for (_, a, _), (_, b, _) in zip(A.parts, B.parts):
            d = bits(a.lat.dd) != bits(b.lat.dd)
            assert not d[:, O.fluid_mask(a.lat.flags)].any()
            assert set(np.unique(a.lat.flags[d.any(axis=0)])) <= {O.FLAG_OBSTACLE}
            # a wall cell stores the sum of what it gathered as its density
            m = O.fluid_mask(a.lat.flags)
            assert n_diff(a.lat.vel, b.lat.vel) == 0 and n_diff(a.lat.rho[m], b.lat.rho[m]) == 0


def test_decomposition_equals_single_domain(oracle_mod):
    """Validate mode (src/main.cpp:309-408): the interior velocity of every
    subdomain equals the matching block of one domain of size
    global - 2*(n-1), bit for bit."""
    O = oracle_mod
    size, nums = (32, 24, 12), (2, 2, 1)
    p = O.Params.lattice(O.cavity_tau(0.1, 30, 1000.0), 0.1, dtype=np.float32)
    A = O.Domain(lambda d: O.OracleKernels("f32"), size, nums, p, "f32")
    A.perturb(SEED, 1e-2)
    red = tuple(s - 2 * (n - 1) for s, n in zip(size, nums))
    S = O.single(O.OracleKernels("f32"), red, p, "f32")
    S.k.perturb(S.lat, (0, 0, 0), red, SEED, 1e-2)
    sx, sy, sz = A.sub
    for _ in range(40):
        A.step()
        S.step()
        for coords, sol, _ in A.parts:
            ox, oy, oz = A.phys_origin(coords)
            loc = sol.lat.vel[:, 1:sz - 1, 1:sy - 1, 1:sx - 1]
            glob = S.lat.vel[:, oz + 1:oz + sz - 1, oy + 1:oy + sy - 1, ox + 1:ox + sx - 1]
            assert n_diff(loc, glob) == 0


def test_minimal_halo_changes_only_ghost_populations(oracle_mod):
    """Exchanging after alpha only the 5 populations the ghost layer's inner
    neighbours gather leaves every fluid and lid cell bit-identical (wall
    cells differ only in the outward, wrap-dependent slots)."""
    O = oracle_mod
    p = O.Params.lattice(O.cavity_tau(0.1, 40, 5000.0), 0.1, 0.17, dtype=np.float32)
    size, nums = (42, 30, 24), (3, 2, 2)
    A = O.Domain(lambda d: O.OracleKernels("f32"), size, nums, p, "f32")
    B = O.Domain(lambda d: O.OracleKernels("f32"), size, nums, p, "f32", halo_mode=1)
    for D in (A, B):
        D.perturb(SEED, 1e-2)
    for _ in range(30):
        A.step()
        B.step()
        for (_, a, _), (_, b, _) in zip(A.parts, B.parts):
            keep = O.fluid_mask(a.lat.flags)
            assert n_diff(a.lat.dd[:, keep], b.lat.dd[:, keep]) == 0
            assert n_diff(a.lat.vel, b.lat.vel) == 0 and n_diff(a.lat.rho[keep], b.lat.rho[keep]) == 0


# ------------------------------------------------------- subgrid model pins
def _np_les_alpha(f, tau0, les_c):
    """Independent float64 statement of one alpha collision with the
    Smagorinsky rate, for fluid cells (no gravity)."""
    from oracle.oracle import E

    e = E.astype(np.float64)
    rho = f.sum(0)
    j = np.einsum("ia,i...->a...", e, f)
    # the reference writes its weights as float literals, also when T = double
    w = np.array([np.float32(1 / 18)] * 4 + [np.float32(1 / 36)] * 12 + [np.float32(1 / 18)] * 2
                 + [np.float32(1 / 3)], dtype=np.float64)
    eu = np.einsum("ia,a...->i...", e, j)
    u2 = (j ** 2).sum(0)
    dp = rho - 1.5 * u2
    feq = w[:, None] * (dp + 3 * eu + 4.5 * eu ** 2)
    # Pi^neq = sum e e f - (rho/3 delta + u u), the incompressible equilibrium's second moment
    third = float(np.float32(1 / 3))  # the constant as the kernels write it, (T)(1.0f/3.0f)
    pi = np.einsum("ia,ib,i...->ab...", e, e, f) - np.einsum("ab,...->ab...", np.eye(3), rho * third) \
        - np.einsum("a...,b...->ab...", j, j)
    q = (pi ** 2).sum((0, 1))
    te = 0.5 * (tau0 + np.sqrt(tau0 ** 2 + les_c * np.sqrt(q)))
    return f + (feq - f) / te


@pytest.mark.parametrize("storage,tol", [("f32", 2e-6), ("f64", 1e-12)])
def test_subgrid_collision_matches_formula(oracle_mod, storage, tol):
    O = oracle_mod
    rdt = O.STORAGE[storage][1]
    dims = (10, 9, 8)
    tau0 = O.cavity_tau(0.1, 64, 20000.0)
    p = O.Params.lattice(tau0, 0.0, cs=0.17, dtype=rdt)
    s = O.Solver(O.OracleKernels(storage), dims, [O.FLAG_OBSTACLE] * 6, p, storage)
    s.k.perturb(s.lat, (0, 0, 0), dims, 99, 5e-2)
    # make the cells non-equilibrium: one beta step, then compare the alpha step
    s.step()
    m = s.lat.flags == O.FLAG_FLUID
    f0 = s.lat.dd[:, m].astype(np.float64)
    s.step()  # alpha: collided populations land in the opposite slots
    got = s.lat.dd[:, m][O.OPP].astype(np.float64)
    want = _np_les_alpha(f0, float(rdt(tau0)), float(rdt(O.les_coefficient(0.17))))
    rel = np.abs(got - want) / np.abs(want)
    assert rel.max() < tol


def _c16_value(code):
    """Value of c16 codes from the format's definition (float64): sign bit 15,
    exponent e = bits 12-14, fraction m = bits 0-11; (1 + m/2^12) 2^(e-12)
    for e > 0, m 2^-23 for e = 0."""
    code = np.asarray(code, dtype=np.int64)
    e, m = (code >> 12) & 7, (code & 0xfff).astype(np.float64)
    mag = np.where(e > 0, (1.0 + m / 4096.0) * np.exp2(e - 12.0), m * 2.0 ** -23)
    return np.where(code & 0x8000, -mag, mag)


def _c16_code(v):
    """c16 code of float32 values from the definition: |v| scaled by 2^-115
    in float (so values below 2^-11 round once, to nearest even, to
    multiples of 2^-34), then rounded to the nearest representable value,
    halves away from zero, saturating at (2 - 2^-12) 2^-5."""
    v = np.asarray(v, dtype=np.float32).astype(np.float64)
    a = np.abs(v)
    small = a < 2.0 ** -11
    a = np.where(small, np.rint(a * 2.0 ** 34) * 2.0 ** -34, a)  # the float scaling's subnormal rounding
    e = np.where(small, 0, np.floor(np.log2(np.maximum(a, 2.0 ** -11))) + 12).astype(np.int64)
    step = np.where(small, 2.0 ** -23, np.exp2(e - 24.0))
    q = np.floor(a / step + 0.5)  # halves away from zero (on the magnitude)
    code = np.where(small, q, (e << 12) + (q - 4096)).astype(np.int64)  # a carry moves into the exponent
    code = np.minimum(code, 0x7fff)
    return (code | np.where(np.signbit(v), 0x8000, 0)).astype(np.uint16)


def _stored_deviation(dd, storage):
    """The stored g_i = f_i - w_i of a shifted lattice, exactly, as float64."""
    if storage == "bf16":
        return (dd.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    if storage == "c16":
        return _c16_value(dd)
    return dd.astype(np.float64)


def _ulp16(x, storage):
    """Spacing of the 16-bit type at x (half precision has subnormals below
    2^-14, c16 below 2^-11)."""
    mant, emin = {"f16": (10, -14), "bf16": (7, -126), "c16": (12, -11)}[storage]
    e = np.maximum(np.floor(np.log2(np.maximum(np.abs(x), 2.0 ** -140))), emin)
    return 2.0 ** (e - mant)


def _c16_raw(oracle):
    import ctypes as C

    L = oracle.lib()
    enc, dec = L.orc_c16_encode_raw, L.orc_c16_decode_raw
    enc.argtypes = dec.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    return enc, dec


def test_c16_format_matches_its_definition(oracle_mod):
    """The oracle's c16 encoder and decoder against the format's definition:
    every one of the 65536 codes decodes to its value and encodes back to
    itself (but -0); random values and exact halves between neighbours, in
    and beyond the range, encode as the definition rounds them."""
    import ctypes as C

    enc, dec = _c16_raw(oracle_mod)
    codes = np.arange(65536, dtype=np.uint16)
    vals = np.empty(65536, np.float32)
    dec(codes.ctypes.data_as(C.c_void_p), vals.ctypes.data_as(C.c_void_p), 65536)
    assert np.array_equal(vals.astype(np.float64), _c16_value(codes))
    back = np.empty(65536, np.uint16)
    enc(vals.ctypes.data_as(C.c_void_p), back.ctypes.data_as(C.c_void_p), 65536)
    keep = codes != 0x8000  # -0 encodes as -0 but +0 and -0 compare equal: skip the pair
    assert np.array_equal(back[keep], codes[keep])
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.uniform(-0.07, 0.07, 200000), rng.uniform(-1e-3, 1e-3, 100000),
                        rng.uniform(-2e-6, 2e-6, 100000), [0.0625, -0.0625, 1.0, -5.0, 2.0 ** -11, 3 * 2.0 ** -24]])
    mid = (_c16_value(codes[1:0x7fff]) + _c16_value(codes[2:0x8000])) / 2  # exact ties between neighbours
    x = np.concatenate([x, mid[np.isfinite(mid)]]).astype(np.float32)
    got = np.empty(x.size, np.uint16)
    enc(x.ctypes.data_as(C.c_void_p), got.ctypes.data_as(C.c_void_p), x.size)
    assert np.array_equal(got, _c16_code(x))


@pytest.mark.parametrize("storage", ["f16", "bf16", "c16"])
@pytest.mark.parametrize("cs", [0.0, 0.17])
def test_deviation_form_collision_matches_formula(oracle_mod, storage, cs):
    """The shifted types collide on deviations with fused multiply-adds; the
    result must be the float64 model of the reference (float weights, the
    incompressible equilibrium, the Smagorinsky rate) up to the rounding of
    the stored value: within one unit in the last place of the 16-bit type."""
    O = oracle_mod
    dims = (10, 9, 8)
    tau0 = O.cavity_tau(0.1, 64, 20000.0)
    p = O.Params.lattice(tau0, 0.0, cs=cs, dtype=np.float32)
    s = O.Solver(O.OracleKernels(storage), dims, [O.FLAG_OBSTACLE] * 6, p, storage)
    s.k.perturb(s.lat, (0, 0, 0), dims, 99, 5e-2)
    s.step()
    m = s.lat.flags == O.FLAG_FLUID
    w = np.array([np.float32(1 / 18)] * 4 + [np.float32(1 / 36)] * 12 + [np.float32(1 / 18)] * 2
                 + [np.float32(1 / 3)], dtype=np.float64)[:, None]
    f0 = _stored_deviation(s.lat.dd[:, m], storage) + w
    s.step()
    got = _stored_deviation(s.lat.dd[:, m][O.OPP], storage)
    if cs:
        want = _np_les_alpha(f0, float(np.float32(tau0)), float(np.float32(O.les_coefficient(cs)))) - w
    else:
        want = _np_les_alpha(f0, float(np.float32(tau0)), 0.0) - w
    assert np.all(np.abs(got - want) <= _ulp16(want, storage))


def test_subgrid_model_off_at_equilibrium(oracle_mod):
    """At equilibrium Pi^neq vanishes, so tau_eff = tau0: one LES step equals
    one plain BGK step with inv_tau = 1/tau0.  The seeded start-up stores
    eq(u) in opposite slots, which an alpha step reads as the equilibrium of
    -u at every cell."""
    O = oracle_mod
    dims = (8, 8, 8)
    tau0 = 0.52
    pl = O.Params.lattice(tau0, 0.0, cs=0.0, dtype=np.float64)
    ls = O.Params.lattice(tau0, 0.0, cs=0.17, dtype=np.float64)
    a = O.Solver(O.OracleKernels("f64"), dims, [O.FLAG_OBSTACLE] * 6, pl, "f64")
    b = O.Solver(O.OracleKernels("f64"), dims, [O.FLAG_OBSTACLE] * 6, ls, "f64")
    for s in (a, b):
        s.k.perturb(s.lat, (0, 0, 0), dims, 5, 1e-2)
        s.lat.counter = 1  # next step is alpha
    a.step()
    b.step()
    np.testing.assert_allclose(a.lat.dd, b.lat.dd, rtol=1e-15, atol=0)


# ------------------------------------------------------------ invariants
def test_rest_state_stays_at_rest(oracle_mod):
    O = oracle_mod
    p = O.Params.lattice(0.6, 0.0, dtype=np.float32)
    s = O.Solver(O.OracleKernels("f32"), (12, 10, 9), [O.FLAG_OBSTACLE] * 6, p, "f32")
    d0 = s.lat.dd.copy()
    for _ in range(20):
        s.step()
    # the float weights do not sum to exactly 1, so rest moves by rounding only
    assert np.max(np.abs(s.lat.dd - d0) / d0) < 1e-6
    assert np.max(np.abs(s.lat.vel)) < 1e-7


def test_closed_box_conserves_mass(oracle_mod):
    """Bounce-back walls and the collision conserve mass up to the weights'
    float rounding, which the reference keeps even for T = double: the total
    over all cells drifts by about 1.5e-8 per step."""
    O = oracle_mod
    dims = (14, 12, 10)
    p = O.Params.lattice(0.55, 0.0, cs=0.17, dtype=np.float64)
    s = O.Solver(O.OracleKernels("f64"), dims, [O.FLAG_OBSTACLE] * 6, p, "f64")
    s.k.perturb(s.lat, (0, 0, 0), dims, 3, 2e-2)
    m0 = s.lat.dd.sum()
    for _ in range(60):
        s.step()
    assert abs(s.lat.dd.sum() - m0) / m0 < 2e-6


@pytest.mark.parametrize("storage,tol", [("f16", 2e-2), ("bf16", 2e-1), ("c16", 5e-3)])
def test_shifted_storage_tracks_f64(oracle_mod, storage, tol):
    """Shifted half/bfloat16 storage against f64 over a short laminar run:
    relative error of the velocity field (RMS over fluid cells)."""
    O = oracle_mod
    dims = (16, 16, 12)
    res = {}
    for st in ("f64", storage):
        p = O.Params.lattice(O.cavity_tau(0.1, 16, 200.0), 0.1, dtype=O.STORAGE[st][1])
        s = O.single(O.OracleKernels(st), dims, p, st)
        for _ in range(60):
            s.step()
        res[st] = s.lat.vel.astype(np.float64)
        m = s.lat.flags == O.FLAG_FLUID
    err = np.sqrt(((res[storage] - res["f64"])[:, m] ** 2).mean()) / np.sqrt((res["f64"][:, m] ** 2).mean())
    assert err < tol


def test_encode_decode_roundtrip(oracle_mod):
    O = oracle_mod
    for st in ("f32", "f64", "f16", "bf16"):
        k = O.OracleKernels(st)
        f = np.random.default_rng(0).uniform(0.0, 0.4, (19, 50)).astype(k.rdt)
        g = k.decode(k.encode(f))
        tol = {"f32": 0, "f64": 0, "f16": 1e-3, "bf16": 1e-2}[st]
        assert np.max(np.abs(g - f)) <= tol * 0.4 + 1e-12


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_per_term_gravity_forcing(oracle_mod, storage):
    """The optional forcing (gravity_mode 1): after one alpha step the change
    against a zero-gravity step is, per opposite pair, +-(coefficient x
    density), and the stored density is the population sum; the default
    mode keeps the reference's chained terms (stored density = last term)."""
    O = oracle_mod
    rdt = O.STORAGE[storage][1]
    dims = (9, 8, 7)
    g = (rdt(2e-4), rdt(-3e-4), rdt(1e-4))
    out = {}
    for mode, grav in ((1, g), (1, (0.0, 0.0, 0.0)), (0, g)):
        p = O.Params.lattice(0.6, 0.0, dtype=rdt, gravity=tuple(float(v) for v in grav), gravity_mode=mode)
        s = O.Solver(O.OracleKernels(storage), dims, [O.FLAG_OBSTACLE] * 6, p, storage)
        s.k.perturb(s.lat, (0, 0, 0), dims, 5, 2e-2)
        rho_in = s.lat.dd.astype(np.float64).sum(0)
        s.lat.counter = 1  # the next step is alpha
        s.step()
        out[(mode, grav == g)] = (s.lat.dd.astype(np.float64), s.lat.rho.astype(np.float64), rho_in)
    m = s.lat.flags == O.FLAG_FLUID
    f_g, rho_g, rho_in = out[(1, True)]
    f_0, _, _ = out[(1, False)]
    gx, gy, gz = (float(v) for v in g)
    w18, w36 = float(np.float32(1 / 18)), float(np.float32(1 / 36))
    coef = [gx * w18, -gy * w18, (gx - gy) * w36, (gx + gy) * w36, (gx + gz) * w36, (gx - gz) * w36,
            (gz - gy) * w36, -(gz + gy) * w36, gz * w18]
    tol = 1e-12 if storage == "f64" else 2e-7
    for k, c in enumerate(coef):
        # alpha writes f_2k into slot 2k+1 and f_2k+1 into slot 2k
        np.testing.assert_allclose((f_g - f_0)[2 * k + 1][m], c * rho_in[m], rtol=1e-5, atol=tol)
        np.testing.assert_allclose((f_g - f_0)[2 * k][m], -c * rho_in[m], rtol=1e-5, atol=tol)
    np.testing.assert_allclose(rho_g[m], rho_in[m], rtol=1e-6)
    _, rho_ref, _ = out[(0, True)]
    assert np.abs(rho_ref[m]).max() < 1e-20  # the reference's chain: the product of nine small terms
