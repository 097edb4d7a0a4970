"""CPU oracle for the D3Q19 hot path: kernels plus the reference host logic.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and the
CPU-baseline arm of bench.py, always as the checker.  The product package never
imports it and has no CPU fallback.

Two interchangeable kernel back-ends drive the same host logic:
  * `OracleKernels`  -- our C restatement (oracle/lbm_oracle.c), built here and
                        on the GPU machine;
  * `RefKernels`     -- the reference's own .cl kernels compiled as C++
                        (oracle/build_ref.py), available only where the
                        reference tree is present.
The host logic restates, in numpy:
  * the step alternation of CLbmSolver::simulationStep
    (src/CLbmSolver.hpp:664-676: even counter -> beta, odd -> alpha);
  * CController::setGeometry, the lid plane (src/CController.hpp:531-546);
  * CManager::initSimulation, boundary flags and CComm geometry per face
    (src/CManager.hpp:78-204);
  * CController::syncAlpha / syncBeta (src/CController.hpp:265-391) with the
    pack/unpack of CLbmSolver::storeDensityDistribution and the masked
    setDensityDistribution (src/CLbmSolver.hpp:695-757), exchanges performed
    face by face in the reference's x, y, z order.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liblbm_oracle.so"

FLAG_OBSTACLE, FLAG_FLUID, FLAG_LID, FLAG_GHOST = 1, 2, 4, 8

# D3Q19 directions, reference order (src/main.cpp:38-66)
E = np.array([(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0),
              (1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0),
              (1, 0, 1), (-1, 0, -1), (1, 0, -1), (-1, 0, 1),
              (0, 1, 1), (0, -1, -1), (0, 1, -1), (0, -1, 1),
              (0, 0, 1), (0, 0, -1), (0, 0, 0)], dtype=np.int64)
OPP = np.array([i ^ 1 if i < 18 else 18 for i in range(19)])

STORAGE = {  # name -> (storage numpy dtype, arithmetic numpy dtype)
    "f32": (np.float32, np.float32),
    "f64": (np.float64, np.float64),
    "f16": (np.float16, np.float32),
    "bf16": (np.uint16, np.float32),
    "c16": (np.uint16, np.float32),
}

_VARIANTS = {"f32": 0, "f64": 1, "f16": 2, "bf16": 3, "c16": 4}


def build(force: bool = False) -> Path:
    """Compile the C restatement (all four storage variants) into one library."""
    src = HERE / "lbm_oracle.c"
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    objs = []
    for name, v in _VARIANTS.items():
        obj = HERE / f"_lbm_oracle_{name}.o"
        subprocess.run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
                        f"-DVARIANT={v}", "-c", str(src), "-o", str(obj)], check=True)
        objs.append(str(obj))
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run(["gcc", "-shared", "-fopenmp", "-o", str(tmp)] + objs + ["-lm"], check=True)
    tmp.replace(LIB)
    for o in objs:
        os.unlink(o)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------------ kernels
class OracleKernels:
    """Our C restatement of the reference kernels (oracle/lbm_oracle.c)."""

    name = "oracle"

    def __init__(self, storage: str = "f32"):
        self.storage = storage
        self.sdt, self.rdt = STORAGE[storage]
        L = lib()
        R = C.c_double if storage == "f64" else C.c_float
        i64, vp, ci = C.c_int64, C.c_void_p, C.c_int
        self._init = getattr(L, f"orc_init_{storage}")
        self._init.argtypes = [vp, vp, vp, vp, vp, i64, i64, i64]
        self._alpha = getattr(L, f"orc_alpha_{storage}")
        self._alpha.argtypes = [vp, vp, vp, vp, i64, i64, i64, R, R, R, R, R, ci, ci, R, R, ci]
        self._beta = getattr(L, f"orc_beta_{storage}")
        self._beta.argtypes = [vp, vp, vp, vp, i64, i64, i64, R, R, R, R, R, ci, ci, R, R, i64]
        self._perturb = getattr(L, f"orc_perturb_{storage}")
        self._perturb.argtypes = [vp, vp, vp, i64, i64, i64, i64, i64, i64, i64, i64, i64, C.c_uint64, C.c_double]
        self._decode = getattr(L, f"orc_decode_{storage}")
        self._decode.argtypes = [vp, vp, i64]
        self._encode = getattr(L, f"orc_encode_{storage}")
        self._encode.argtypes = [vp, vp, i64]

    def init(self, lat: "Lattice", bc):
        bc = np.ascontiguousarray(bc, dtype=np.int32)
        self._init(_ptr(lat.dd), _ptr(lat.flags), _ptr(lat.vel), _ptr(lat.rho), _ptr(bc), *lat.dims)

    def alpha(self, lat: "Lattice", p: "Params"):
        self._alpha(_ptr(lat.dd), _ptr(lat.flags), _ptr(lat.vel), _ptr(lat.rho), *lat.dims,
                    p.inv_tau, *p.gravity, p.lid, int(p.store_vel), int(p.store_rho), p.tau0, p.les_c,
                    int(p.gravity_mode))

    def beta(self, lat: "Lattice", p: "Params"):
        self._beta(_ptr(lat.dd), _ptr(lat.flags), _ptr(lat.vel), _ptr(lat.rho), *lat.dims,
                   p.inv_tau, *p.gravity, p.lid, int(p.store_vel), int(p.store_rho), p.tau0, p.les_c, p.wg)

    def perturb(self, lat: "Lattice", origin, phys, seed: int, amp: float):
        self._perturb(_ptr(lat.dd), _ptr(lat.vel), _ptr(lat.rho), *lat.dims, *origin, *phys, seed, amp)

    def decode(self, dd: np.ndarray) -> np.ndarray:
        out = np.empty(dd.shape, dtype=self.rdt)
        self._decode(_ptr(np.ascontiguousarray(dd)), _ptr(out), dd[0].size)
        return out

    def encode(self, f: np.ndarray) -> np.ndarray:
        out = np.empty(f.shape, dtype=self.sdt)
        self._encode(_ptr(np.ascontiguousarray(f, dtype=self.rdt)), _ptr(out), f[0].size)
        return out


class RefKernels:
    """The reference's own src/cl_programs kernels compiled as C++.

    Built per (T, X, Y, Z, work-group size) by oracle/build_ref.py; only where
    the reference tree is present.  The work-group size is the reference
    default of 128 (`kernel-count`, conf.xml and src/main.cpp:114)."""

    name = "reference"

    def __init__(self, storage: str, nx: int, ny: int, nz: int, wg: int = 128):
        from . import build_ref  # noqa: local import, optional dependency

        if storage not in ("f32", "f64"):
            raise ValueError("reference kernels exist in f32/f64 only")
        self.storage, self.wg = storage, wg
        self.sdt, self.rdt = STORAGE[storage]
        self.dims = (nx, ny, nz)
        L = C.CDLL(str(build_ref.build(storage, nx, ny, nz, wg)))
        R = C.c_double if storage == "f64" else C.c_float
        vp, ci = C.c_void_p, C.c_int
        self._init = L.ref_init
        self._init.argtypes = [vp, vp, vp, vp, vp, R]
        self._alpha = L.ref_alpha
        self._alpha.argtypes = [vp, vp, vp, vp, R, R, R, R, R]
        self._beta = L.ref_beta
        self._beta.argtypes = [vp, vp, vp, vp, R, R, R, R, R]
        self._beta.restype = ci
        self._copy = L.ref_copy_rect
        self._copy.argtypes = [vp] + [ci] * 7 + [vp] + [ci] * 7 + [ci] * 3

    def _check(self, lat):
        if tuple(lat.dims) != self.dims:
            raise ValueError("reference kernels are compiled for another size")
        if not (lat.store_vel and lat.store_rho):
            raise ValueError("reference build always stores velocity and density")

    def init(self, lat, bc):
        self._check(lat)
        bc = np.ascontiguousarray(bc, dtype=np.int32)
        self._init(_ptr(lat.dd), _ptr(lat.flags), _ptr(lat.vel), _ptr(lat.rho), _ptr(bc), 0.0)

    def perturb(self, lat, origin, phys, seed, amp):
        """The seeded start-up field is an input generator, not a reference
        kernel: both back-ends receive the buffer the C oracle writes."""
        OracleKernels(self.storage).perturb(lat, origin, phys, seed, amp)

    def alpha(self, lat, p):
        self._check(lat)
        if p.les_c != 0:
            raise ValueError("the reference has no subgrid model")
        if p.gravity_mode:
            raise ValueError("the reference has only its own (aliased) gravity terms")
        self._alpha(_ptr(lat.dd), _ptr(lat.flags), _ptr(lat.vel), _ptr(lat.rho), p.inv_tau, *p.gravity, p.lid)

    def beta(self, lat, p):
        self._check(lat)
        if p.les_c != 0:
            raise ValueError("the reference has no subgrid model")
        if self._beta(_ptr(lat.dd), _ptr(lat.flags), _ptr(lat.vel), _ptr(lat.rho), p.inv_tau, *p.gravity, p.lid):
            raise ValueError("cell count must be a multiple of the work-group size")


# -------------------------------------------------------------- host logic
@dataclass
class Params:
    """Kernel arguments (src/CLbmSolver.hpp:593-612) plus the subgrid model.

    les_c = 18*sqrt(2)*Cs^2 (0 turns the model off) and tau0 = 1/inv_tau is
    the molecular relaxation time.  wg selects the reference beta kernel's
    work-group realignment semantics in the C oracle (0 = plain linear wrap).
    gravity_mode 1 is the optional per-term forcing (not the reference's)."""

    inv_tau: float
    tau0: float = 0.0
    les_c: float = 0.0
    gravity: tuple = (0.0, 0.0, 0.0)
    lid: float = 0.0
    store_vel: bool = True
    store_rho: bool = True
    wg: int = 0
    gravity_mode: int = 0

    @staticmethod
    def lattice(tau: float, lid: float, cs: float = 0.0, dtype=np.float32, **kw) -> "Params":
        """Parameters from lattice units; values rounded to the arithmetic type."""
        t = dtype(tau)
        return Params(inv_tau=float(dtype(1) / t), tau0=float(t), les_c=float(dtype(les_coefficient(cs))),
                      lid=float(dtype(lid)), **kw)


def les_coefficient(cs: float) -> float:
    """C = 18*sqrt(2)*Cs^2 of tau_eff = (tau0 + sqrt(tau0^2 + C*sqrt(Q)))/2."""
    return 18.0 * math.sqrt(2.0) * cs * cs


def cavity_tau(u: float, length: float, re: float) -> float:
    """tau = 3 nu + 1/2 with nu = U L / Re (lattice units)."""
    return 3.0 * u * length / re + 0.5


@dataclass
class Lattice:
    dims: tuple
    storage: str = "f32"
    store_vel: bool = True
    store_rho: bool = True
    counter: int = 0
    dd: np.ndarray = field(default=None, repr=False)
    flags: np.ndarray = field(default=None, repr=False)
    vel: np.ndarray = field(default=None, repr=False)
    rho: np.ndarray = field(default=None, repr=False)

    def __post_init__(self):
        nx, ny, nz = self.dims
        sdt, rdt = STORAGE[self.storage]
        self.dd = np.zeros((19, nz, ny, nx), sdt)
        self.flags = np.zeros((nz, ny, nx), np.int32)
        self.vel = np.zeros((3, nz, ny, nx), rdt)
        self.rho = np.zeros((nz, ny, nx), rdt)


def region(origin, size):
    """numpy index of a (x,y,z) box in a (..., z, y, x) array."""
    (ox, oy, oz), (sx, sy, sz) = origin, size
    return (slice(oz, oz + sz), slice(oy, oy + sy), slice(ox, ox + sx))


class Solver:
    """One subdomain: the CLbmSolver host logic over a kernel back-end."""

    def __init__(self, kernels, dims, bc, params: Params, storage="f32"):
        self.k = kernels
        self.p = params
        self.bc = np.asarray(bc, dtype=np.int32).reshape(6)
        self.lat = Lattice(tuple(dims), storage, params.store_vel, params.store_rho)
        self.reset()

    def reset(self):
        """src/CLbmSolver.hpp:619-635"""
        self.lat.counter = 0
        self.k.init(self.lat, self.bc)

    def step(self):
        """src/CLbmSolver.hpp:664-676: odd counter -> alpha, even -> beta."""
        if self.lat.counter & 1:
            self.k.alpha(self.lat, self.p)
        else:
            self.k.beta(self.lat, self.p)
        self.lat.counter += 1

    def set_geometry(self):
        """Lid plane y = Y-2, x in [1, X-2], z in [1, Z-2]: src/CController.hpp:531-546."""
        nx, ny, nz = self.lat.dims
        self.lat.flags[region((1, ny - 2, 1), (nx - 2, 1, nz - 2))] = FLAG_LID


@dataclass
class Comm:
    """CComm (src/CComm.hpp:20-77): one face exchange with subdomain dst."""

    dst: int
    send_size: tuple
    recv_size: tuple
    send_origin: tuple
    recv_origin: tuple
    direction: tuple
    axis: int


def manager_layout(size, nums):
    """CManager::setSubdomainNums + initSimulation (src/CManager.hpp:49-204).

    Returns, per subdomain id, (coords, BC[6], [Comm...], has_lid)."""
    size, nums = tuple(size), tuple(nums)
    if any(s % n for s, n in zip(size, nums)):
        raise ValueError("Number of subdomains does not match with the grid size!")
    sub = tuple(s // n for s, n in zip(size, nums))
    out = []
    for sid in range(nums[0] * nums[1] * nums[2]):
        c = (sid % nums[0], (sid // nums[0]) % nums[1], sid // (nums[0] * nums[1]))
        bc = [FLAG_GHOST] * 6
        for a in range(3):
            if c[a] == 0:
                bc[2 * a] = FLAG_OBSTACLE
            if c[a] == nums[a] - 1:
                bc[2 * a + 1] = FLAG_OBSTACLE
        comms = []
        stride = (1, nums[0], nums[0] * nums[1])
        for a in range(3):
            face = list(sub)
            face[a] = 1
            for upper in (0, 1):
                if bc[2 * a + upper] != FLAG_GHOST:
                    continue
                so, ro, d = [0, 0, 0], [0, 0, 0], [0, 0, 0]
                so[a] = sub[a] - 2 if upper else 1
                ro[a] = sub[a] - 1 if upper else 0
                d[a] = -1 if upper else 1
                comms.append(Comm(sid + (stride[a] if upper else -stride[a]), tuple(face), tuple(face),
                                  tuple(so), tuple(ro), tuple(d), a))
        out.append((c, bc, comms, c[1] == nums[1] - 1))
    return sub, out


class Domain:
    """All subdomains of one run in one process: CManager + CController.

    `kernels_for(dims)` returns a kernel back-end for a subdomain size."""

    def __init__(self, kernels_for, size, nums, params: Params, storage="f32", lid_geometry=True, halo_mode=0):
        self.p = params
        self.halo_mode = halo_mode  # 1: after alpha only the populations gathered inward
        self.sub, layout = manager_layout(size, nums)
        self.nums = tuple(nums)
        self.parts = []
        for coords, bc, comms, has_lid in layout:
            s = Solver(kernels_for(self.sub), self.sub, bc, params, storage)
            if has_lid and lid_geometry:
                s.set_geometry()
            self.parts.append((coords, s, comms))

    @property
    def counter(self):
        return self.parts[0][1].lat.counter

    def phys_origin(self, coords):
        """Physical origin of a subdomain: neighbours overlap by two cells."""
        return tuple(c * (s - 2) for c, s in zip(coords, self.sub))

    def phys_size(self):
        return tuple(n * (s - 2) + 2 for n, s in zip(self.nums, self.sub))

    def perturb(self, seed: int, amp: float):
        for coords, s, _ in self.parts:
            s.k.perturb(s.lat, self.phys_origin(coords), self.phys_size(), seed, amp)

    def step(self):
        """CController::computeNextStep for every subdomain (src/CController.hpp:385-391)."""
        for _, s, _ in self.parts:
            s.step()
        if self.counter & 1:
            self._sync(beta=True)
        else:
            self._sync(beta=False)

    def _sync(self, beta: bool):
        """syncAlpha / syncBeta over all subdomains, face by face in x, y, z order.

        Within one axis the sent regions and the received regions of every
        subdomain are disjoint, so packing all sends of an axis before
        unpacking them equals the reference's pairwise MPI exchanges."""
        for axis in range(3):
            packets = {}
            for sid, (_, s, comms) in enumerate(self.parts):
                for cm in comms:
                    if cm.axis != axis:
                        continue
                    if beta:   # ghost layer goes back to its owner (src/CController.hpp:333-337)
                        origin, size = cm.recv_origin, cm.recv_size
                    else:
                        origin, size = cm.send_origin, cm.send_size
                    packets[(sid, cm.dst)] = s.lat.dd[(slice(None),) + region(origin, size)].copy()
            for sid, (_, s, comms) in enumerate(self.parts):
                for cm in comms:
                    if cm.axis != axis:
                        continue
                    buf = packets[(cm.dst, sid)]
                    if beta:   # unpack into the inner layer, inward populations only
                        sel = [f for f in range(19) if int(np.dot(cm.direction, E[f])) > 0]
                        s.lat.dd[(sel,) + region(cm.send_origin, cm.send_size)] = buf[sel]
                    elif self.halo_mode:  # the ghost populations the inner neighbours gather
                        sel = [f for f in range(19) if int(np.dot(cm.direction, E[f])) < 0]
                        s.lat.dd[(sel,) + region(cm.recv_origin, cm.recv_size)] = buf[sel]
                    else:
                        s.lat.dd[(slice(None),) + region(cm.recv_origin, cm.recv_size)] = buf


def single(kernels, dims, params: Params, storage="f32", lid=True) -> Solver:
    """A one-subdomain cavity: walls on all six faces plus the lid plane."""
    s = Solver(kernels, dims, [FLAG_OBSTACLE] * 6, params, storage)
    if lid:
        s.set_geometry()
    return s


def fluid_mask(flags: np.ndarray) -> np.ndarray:
    """Cells whose every population is defined independent of the wrap rules."""
    return (flags == FLAG_FLUID) | (flags == FLAG_LID)
