"""ctypes binding of liblbm_gb300.so -- the C ABI declared in include/lbm_gb300.h.

The library must have been built for sm_103a (``build.build()``); there is no
CPU fallback: loading fails loudly when the library is missing, and every
call that fails raises ``LbmError`` with the library's message.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

from .build import LIB

F32, F64, F16, BF16, C16 = 0, 1, 2, 3, 4
STORAGE_NAMES = {"f32": F32, "f64": F64, "f16": F16, "bf16": BF16, "c16": C16}
FIELD_DD, FIELD_VELOCITY, FIELD_DENSITY, FIELD_FLAGS = 0, 1, 2, 3
FLAG_OBSTACLE, FLAG_FLUID, FLAG_VELOCITY_INJECTION, FLAG_GHOST_LAYER = 1, 2, 4, 8


class LbmError(RuntimeError):
    pass


class Cavity(C.Structure):
    """lbm_cavity: one lid-driven cavity of an ensemble (lattice units)."""

    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("storage", C.c_int),
                ("tau0", C.c_double), ("cs", C.c_double), ("lid", C.c_double), ("steps", C.c_int64),
                ("seed", C.c_uint64), ("amp", C.c_double)]

    @staticmethod
    def make(dims, storage=0, tau0=0.6, cs=0.0, lid=0.05, steps=100, seed=0, amp=0.0):
        c = Cavity()
        c.nx, c.ny, c.nz = (int(x) for x in dims)
        c.storage, c.tau0, c.cs, c.lid, c.steps, c.seed, c.amp = storage, tau0, cs, lid, int(steps), seed, amp
        return c


class Params(C.Structure):
    """lbm_params: kernel arguments in double (rounded to the arithmetic type by the library)."""

    _fields_ = [("inv_tau", C.c_double), ("tau0", C.c_double), ("les_c", C.c_double),
                ("gravity", C.c_double * 3), ("lid", C.c_double), ("gravity_mode", C.c_int32)]

    @staticmethod
    def make(inv_tau: float, tau0: float = 0.0, les_c: float = 0.0, gravity=(0.0, 0.0, 0.0), lid: float = 0.0,
             gravity_mode: int = 0):
        p = Params()
        p.inv_tau, p.tau0, p.les_c, p.lid, p.gravity_mode = inv_tau, tau0, les_c, lid, gravity_mode
        for a in range(3):
            p.gravity[a] = gravity[a]
        return p


def les_coefficient(cs: float) -> float:
    """18*sqrt(2)*Cs^2 of the subgrid relaxation time."""
    return 18.0 * math.sqrt(2.0) * cs * cs


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not Path(LIB).exists():
        raise LbmError(f"{LIB} is not built: run `python -m turbulent_lbm_multigpu_gb300.build` "
                       "(CUDA toolkit, sm_103a); there is no CPU fallback")
    L = C.CDLL(str(LIB))
    vp, ci, i64, u64, cd = C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_double
    ip = C.POINTER(C.c_int)
    sig = {
        "lbm_cu_last_error": ([], C.c_char_p),
        "lbm_cu_version": ([], C.c_char_p),
        "lbm_cu_synchronize": ([vp], ci),
        "lbm_cu_check_wait_timeout": ([C.c_uint, vp], ci),
        "lbm_cu_create": ([ci, ci, ci, ci, ci, ci, C.POINTER(vp)], ci),
        "lbm_cu_destroy": ([vp], ci),
        "lbm_cu_dims": ([vp, ip], ci),
        "lbm_cu_set_params": ([vp, C.POINTER(Params)], ci),
        "lbm_cu_init": ([vp, ip, vp], ci),
        "lbm_cu_perturb": ([vp, ip, ip, u64, cd, vp], ci),
        "lbm_cu_step": ([vp, ci, vp], ci),
        "lbm_cu_set_kernel_shape": ([vp, ci], ci),
        "lbm_cu_set_fp64_contraction": ([vp, ci], ci),
        "lbm_cu_domain_set_fp64_contraction": ([vp, ci], ci),
        "lbm_cu_domain_set_fused_exchange": ([vp, ci], ci),
        "lbm_cu_read": ([vp, ci, ip, ip, vp, vp], ci),
        "lbm_cu_write": ([vp, ci, ip, ip, vp, ip, vp], ci),
        "lbm_cu_halo": ([vp, ip, vp, ip, ip, ip, vp], ci),
        "lbm_cu_reduce_conserved": ([vp, ci, C.POINTER(cd), vp], ci),
        "lbm_cu_reduce_conserved_noalloc": ([vp, ci, C.POINTER(cd), vp], ci),
        "lbm_cu_compare_velocity": ([vp, ci, vp, ci, C.POINTER(cd), vp], ci),
        "lbm_cu_deviation_stats": ([vp, C.POINTER(cd), vp], ci),
        "lbm_cu_domain_create": ([ip, ip, ci, ci, ci, ci, C.POINTER(vp)], ci),
        "lbm_cu_domain_destroy": ([vp], ci),
        "lbm_cu_domain_wrap": ([C.POINTER(vp), ip, ip, ci, C.POINTER(vp)], ci),
        "lbm_cu_domain_set_counter": ([vp, i64], ci),
        "lbm_cu_domain_set_params": ([vp, C.POINTER(Params)], ci),
        "lbm_cu_domain_reset": ([vp, vp], ci),
        "lbm_cu_domain_perturb": ([vp, u64, cd, vp], ci),
        "lbm_cu_domain_run": ([vp, ci, ci, vp], ci),
        "lbm_cu_domain_counter": ([vp, C.POINTER(i64)], ci),
        "lbm_cu_domain_set_store_interval": ([vp, ci], ci),
        "lbm_cu_domain_set_halo_mode": ([vp, ci], ci),
        "lbm_cu_domain_set_kernel_shape": ([vp, ci], ci),
        "lbm_cu_domain_profile": ([vp, ci], ci),
        "lbm_cu_domain_kernel_time": ([vp, C.POINTER(cd), C.POINTER(i64), ci], ci),
        "lbm_cu_domain_prepare_timed_run": ([vp, ci, ci, vp], ci),
        "lbm_cu_domain_kernel_time_by_step": ([vp, C.POINTER(cd), C.POINTER(i64), ci], ci),
        "lbm_cu_domain_subdomains": ([vp, ip, ip], ci),
        "lbm_cu_domain_lattice": ([vp, ci], vp),
        "lbm_cu_run": ([vp, i64, i64, vp], ci),
        "lbm_cu_checkpoint_save": ([vp, C.c_char_p, i64, vp], ci),
        "lbm_cu_checkpoint_load": ([vp, C.c_char_p, C.POINTER(i64), vp], ci),
        "lbm_cu_domain_checkpoint_save": ([vp, C.c_char_p, vp], ci),
        "lbm_cu_domain_checkpoint_load": ([vp, C.c_char_p, vp], ci),
        "lbm_cu_batch_create": ([C.POINTER(Cavity), ci, ci, C.POINTER(vp)], ci),
        "lbm_cu_batch_destroy": ([vp], ci),
        "lbm_cu_batch_reset": ([vp, vp], ci),
        "lbm_cu_batch_set_kernel_shape": ([vp, ci], ci),
        "lbm_cu_batch_tune": ([vp, ci, ip, C.POINTER(cd), vp], ci),
        "lbm_cu_batch_run": ([vp, i64, ci, vp], ci),
        "lbm_cu_batch_status": ([vp, C.POINTER(i64), ip], ci),
        "lbm_cu_batch_lattice": ([vp, ci], vp),
        "lbm_cu_server_create": ([cd, ci, ci, C.POINTER(vp)], ci),
        "lbm_cu_server_destroy": ([vp], ci),
        "lbm_cu_server_set_kernel_shape": ([vp, ci], ci),
        "lbm_cu_server_submit": ([vp, C.POINTER(Cavity), C.POINTER(i64)], ci),
        "lbm_cu_server_tick": ([vp, i64, ci, ip, vp], ci),
        "lbm_cu_server_poll": ([vp, C.POINTER(i64), ci, ip], ci),
        "lbm_cu_server_lattice": ([vp, i64], vp),
        "lbm_cu_server_release": ([vp, i64], ci),
        "lbm_cu_server_status": ([vp, ip, ip, C.POINTER(cd), C.POINTER(i64)], ci),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def check(rc: int):
    if rc != 0:
        raise LbmError(lib().lbm_cu_last_error().decode())


def ivec(v):
    if v is None:
        return None
    return (C.c_int * len(v))(*[int(x) for x in v])


def real_dtype(storage: int):
    return np.float64 if storage == F64 else np.float32


class Lattice:
    """One lattice (subdomain) on the current GPU, owning its device fields."""

    def __init__(self, nx, ny, nz, storage=F32, store_velocity=True, store_density=True, handle=None, owner=None):
        self.dims = (int(nx), int(ny), int(nz))
        self.storage = storage
        self.store_velocity, self.store_density = bool(store_velocity), bool(store_density)
        self._owner = owner
        if handle is None:
            h = C.c_void_p()
            check(lib().lbm_cu_create(nx, ny, nz, storage, int(store_velocity), int(store_density), C.byref(h)))
            self.h = h
        else:
            self.h = C.c_void_p(handle)

    def close(self):
        if self._owner is None and self.h:
            lib().lbm_cu_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def cells(self):
        return self.dims[0] * self.dims[1] * self.dims[2]

    def set_params(self, p: Params):
        check(lib().lbm_cu_set_params(self.h, C.byref(p)))

    def init(self, bc, stream=None):
        check(lib().lbm_cu_init(self.h, ivec(bc), stream))

    def perturb(self, origin, phys, seed, amp, stream=None):
        check(lib().lbm_cu_perturb(self.h, ivec(origin), ivec(phys), seed, amp, stream))

    def step(self, parity: int, stream=None):
        check(lib().lbm_cu_step(self.h, parity, stream))

    def set_kernel_shape(self, cells_per_thread: int):
        check(lib().lbm_cu_set_kernel_shape(self.h, cells_per_thread))

    def set_fp64_contraction(self, enable: bool):
        """Double storage: fused multiply-adds in the step (1e-15 per step off the reference arithmetic)."""
        check(lib().lbm_cu_set_fp64_contraction(self.h, int(enable)))

    def _shape(self, field, size):
        sx, sy, sz = size
        planes = {FIELD_DD: 19, FIELD_VELOCITY: 3, FIELD_DENSITY: 1, FIELD_FLAGS: 1}[field]
        dt = np.int32 if field == FIELD_FLAGS else real_dtype(self.storage)
        return (planes, sz, sy, sx), dt

    def read(self, field, origin=None, size=None, out=None, stream=None):
        size = tuple(size) if size is not None else self.dims
        shape, dt = self._shape(field, size)
        if out is None:
            out = np.empty(shape, dt)
        if out.dtype != dt or out.size != int(np.prod(shape)) or not out.flags.c_contiguous:
            raise LbmError(f"host buffer must be a contiguous {dt.__name__} array of {int(np.prod(shape))} elements")
        check(lib().lbm_cu_read(self.h, field, ivec(origin), ivec(size), out.ctypes.data_as(C.c_void_p), stream))
        return out

    def write(self, field, src, origin=None, size=None, norm=None, stream=None):
        size = tuple(size) if size is not None else self.dims
        shape, dt = self._shape(field, size)
        src = np.ascontiguousarray(src, dtype=dt)
        if src.size != int(np.prod(shape)):
            raise LbmError(f"host buffer must hold {int(np.prod(shape))} elements")
        check(lib().lbm_cu_write(self.h, field, ivec(origin), ivec(size), src.ctypes.data_as(C.c_void_p),
                                 ivec(norm), stream))

    def run(self, first_step: int, steps: int, stream=None):
        """`steps` steps, one launch each, starting at step counter `first_step`."""
        check(lib().lbm_cu_run(self.h, first_step, steps, stream))

    def reduce_conserved(self, layout: int, stream=None):
        out = (C.c_double * 5)()
        check(lib().lbm_cu_reduce_conserved(self.h, layout, out, stream))
        return np.array(out[:], dtype=np.float64)

    def checkpoint_save(self, path, counter: int, stream=None):
        """Raw populations, flags and the step counter to a file (restart is bit-exact)."""
        check(lib().lbm_cu_checkpoint_save(self.h, str(path).encode(), int(counter), stream))

    def checkpoint_load(self, path, stream=None) -> int:
        """Restore a checkpoint of a lattice of the same size and storage; returns its step counter."""
        c = C.c_int64()
        check(lib().lbm_cu_checkpoint_load(self.h, str(path).encode(), C.byref(c), stream))
        return c.value

    def reduce_conserved_noalloc(self, layout: int, stream=None):
        """The same sums without any device allocation (fixed in-library
        scratch, lattices up to 512^3 cells); see include/lbm_gb300.h."""
        out = (C.c_double * 5)()
        check(lib().lbm_cu_reduce_conserved_noalloc(self.h, layout, out, stream))
        return np.array(out[:], dtype=np.float64)


def deviation_stats(L: Lattice, stream=None):
    """{values, zero, subnormal, saturated, max_abs} of a 16-bit lattice's stored deviations (fluid cells)."""
    out = (C.c_double * 5)()
    check(lib().lbm_cu_deviation_stats(L.h, out, stream))
    n, z, sub, sat, mx = out[:]
    return {"values": int(n), "zero": int(z), "subnormal": int(sub), "saturated": int(sat), "max_abs": mx,
            "subnormal_fraction": sub / n if n else 0.0, "zero_fraction": z / n if n else 0.0}


def compare_velocity(a: Lattice, layout_a: int, b: Lattice, layout_b: int, stream=None):
    """{max_abs, rms, rel_rms, rel_max, cells} of a's velocity against b's over a's fluid cells."""
    out = (C.c_double * 5)()
    check(lib().lbm_cu_compare_velocity(a.h, layout_a, b.h, layout_b, out, stream))
    mx, se, sr, mr, n = out[:]
    n = max(n, 1.0)
    return {"max_abs": mx, "rms": math.sqrt(se / n), "rel_rms": math.sqrt(se / sr) if sr > 0 else 0.0,
            "rel_max": mx / mr if mr > 0 else 0.0, "ref_rms": math.sqrt(sr / n), "ref_max": mr, "cells": int(n)}


def halo(src: Lattice, src_origin, dst: Lattice, dst_origin, size, norm=None, stream=None):
    check(lib().lbm_cu_halo(src.h, ivec(src_origin), dst.h, ivec(dst_origin), ivec(size), ivec(norm), stream))


def synchronize(stream=None):
    """Wait for the stream (None: the device); raises LbmError if a staged
    kernel gave up waiting for its bulk copies since the last call."""
    check(lib().lbm_cu_synchronize(stream))


def check_wait_timeout(polls=1 << 12, stream=None):
    """Launch the bounded-wait check: its wait runs out by design and the
    next synchronize() reports it."""
    check(lib().lbm_cu_check_wait_timeout(polls, stream))


class Domain:
    """A decomposed domain on one GPU (CManager + CController, device-local halos)."""

    def __init__(self, size, nums, storage=F32, store_velocity=False, store_density=False, lid_geometry=True):
        self.size, self.nums = tuple(size), tuple(nums)
        self.storage = storage
        h = C.c_void_p()
        check(lib().lbm_cu_domain_create(ivec(size), ivec(nums), storage, int(store_velocity), int(store_density),
                                         int(lid_geometry), C.byref(h)))
        self.h = h
        cnt = C.c_int()
        sub = (C.c_int * 3)()
        check(lib().lbm_cu_domain_subdomains(self.h, C.byref(cnt), sub))
        self.sub = tuple(sub[:])
        self.subdomains = [Lattice(*self.sub, storage, store_velocity, store_density,
                                   handle=lib().lbm_cu_domain_lattice(self.h, i), owner=self) for i in range(cnt.value)]

    def close(self):
        if self.h:
            lib().lbm_cu_domain_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def cells(self):
        return self.size[0] * self.size[1] * self.size[2]

    def set_params(self, p: Params):
        check(lib().lbm_cu_domain_set_params(self.h, C.byref(p)))

    def reset(self, stream=None):
        check(lib().lbm_cu_domain_reset(self.h, stream))

    def perturb(self, seed, amp, stream=None):
        check(lib().lbm_cu_domain_perturb(self.h, seed, amp, stream))

    def run(self, steps, use_graph=True, stream=None):
        check(lib().lbm_cu_domain_run(self.h, steps, int(use_graph), stream))

    @classmethod
    def wrap(cls, lattices, size, nums, lid_geometry=True):
        """A view over lattices the caller owns and initialised, one per
        subdomain in subdomain order (lbm_cu_domain_wrap)."""
        self = cls.__new__(cls)
        self.size, self.nums = tuple(size), tuple(nums)
        self.storage = lattices[0].storage
        arr = (C.c_void_p * len(lattices))(*[L.h.value for L in lattices])
        h = C.c_void_p()
        check(lib().lbm_cu_domain_wrap(arr, ivec(size), ivec(nums), int(lid_geometry), C.byref(h)))
        self.h = h
        self.sub = lattices[0].dims
        self.subdomains = list(lattices)
        return self

    @property
    def counter(self):
        c = C.c_int64()
        check(lib().lbm_cu_domain_counter(self.h, C.byref(c)))
        return c.value

    @counter.setter
    def counter(self, value):
        check(lib().lbm_cu_domain_set_counter(self.h, int(value)))

    def set_store_interval(self, interval: int):
        check(lib().lbm_cu_domain_set_store_interval(self.h, interval))

    def checkpoint_save(self, path, stream=None):
        check(lib().lbm_cu_domain_checkpoint_save(self.h, str(path).encode(), stream))

    def checkpoint_load(self, path, stream=None):
        """Restore every subdomain and the step counter."""
        check(lib().lbm_cu_domain_checkpoint_load(self.h, str(path).encode(), stream))

    def set_kernel_shape(self, cells_per_thread: int):
        check(lib().lbm_cu_domain_set_kernel_shape(self.h, cells_per_thread))

    def set_fp64_contraction(self, enable: bool):
        check(lib().lbm_cu_domain_set_fp64_contraction(self.h, int(enable)))

    def set_fused_exchange(self, enable: bool):
        """One-cell alpha steps do the x part of the exchange after them (default on)."""
        check(lib().lbm_cu_domain_set_fused_exchange(self.h, int(enable)))

    def set_halo_mode(self, mode: int):
        """0: all 19 populations after alpha (reference); 1: the 5 read inward."""
        check(lib().lbm_cu_domain_set_halo_mode(self.h, mode))

    def profile(self, enable: bool):
        check(lib().lbm_cu_domain_profile(self.h, int(enable)))

    def kernel_time(self, reset=False):
        ms, n = C.c_double(), C.c_int64()
        check(lib().lbm_cu_domain_kernel_time(self.h, C.byref(ms), C.byref(n), int(reset)))
        return ms.value, n.value

    def kernel_time_by_step(self, reset=False):
        """((beta ms, launches), (alpha ms, launches)) of the timed step kernels."""
        ms, n = (C.c_double * 2)(), (C.c_int64 * 2)()
        check(lib().lbm_cu_domain_kernel_time_by_step(self.h, ms, n, int(reset)))
        return (ms[0], n[0]), (ms[1], n[1])

    def prepare_timed_run(self, steps, every=1, stream=None):
        """Capture the next `steps` steps as one graph with events around the
        step kernels of steps k % every < 2 (run it with run(steps,
        use_graph=True) while profiling)."""
        check(lib().lbm_cu_domain_prepare_timed_run(self.h, int(steps), int(every), stream))


class Batch:
    """An ensemble of cavities advanced together (lbm_cu_batch_*)."""

    def __init__(self, cavities, store_velocity=True):
        arr = (Cavity * len(cavities))(*cavities)
        h = C.c_void_p()
        check(lib().lbm_cu_batch_create(arr, len(cavities), int(store_velocity), C.byref(h)))
        self.h = h
        self.cavities = list(cavities)
        self.lattices = [Lattice(c.nx, c.ny, c.nz, c.storage, store_velocity, False,
                                 handle=lib().lbm_cu_batch_lattice(self.h, i), owner=self)
                         for i, c in enumerate(self.cavities)]

    def close(self):
        if self.h:
            lib().lbm_cu_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self, stream=None):
        check(lib().lbm_cu_batch_reset(self.h, stream))

    def set_kernel_shape(self, cells_per_thread):
        check(lib().lbm_cu_batch_set_kernel_shape(self.h, cells_per_thread))

    def tune(self, trial_steps=20, stream=None):
        shape, ms = C.c_int(), C.c_double()
        check(lib().lbm_cu_batch_tune(self.h, trial_steps, C.byref(shape), C.byref(ms), stream))
        return shape.value, ms.value

    def run(self, max_steps=-1, use_graph=True, stream=None):
        check(lib().lbm_cu_batch_run(self.h, max_steps, int(use_graph), stream))

    def status(self):
        done, active = C.c_int64(), C.c_int()
        check(lib().lbm_cu_batch_status(self.h, C.byref(done), C.byref(active)))
        return done.value, active.value


class Server:
    """Continuous-batching solve server (lbm_cu_server_*)."""

    def __init__(self, hbm_budget_bytes, max_active=0, store_velocity=True):
        h = C.c_void_p()
        check(lib().lbm_cu_server_create(float(hbm_budget_bytes), max_active, int(store_velocity), C.byref(h)))
        self.h = h
        self.store_velocity = store_velocity
        self.specs = {}

    def close(self):
        if self.h:
            lib().lbm_cu_server_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_kernel_shape(self, cells_per_thread):
        check(lib().lbm_cu_server_set_kernel_shape(self.h, cells_per_thread))

    def submit(self, cavity: Cavity) -> int:
        i = C.c_int64()
        check(lib().lbm_cu_server_submit(self.h, C.byref(cavity), C.byref(i)))
        self.specs[i.value] = cavity
        return i.value

    def tick(self, max_steps=-1, use_graph=True, stream=None) -> int:
        adm = C.c_int()
        check(lib().lbm_cu_server_tick(self.h, max_steps, int(use_graph), C.byref(adm), stream))
        return adm.value

    def poll(self, capacity=4096):
        ids = (C.c_int64 * capacity)()
        n = C.c_int()
        check(lib().lbm_cu_server_poll(self.h, ids, capacity, C.byref(n)))
        return list(ids[:n.value])

    def lattice(self, sid) -> Lattice:
        c = self.specs[sid]
        h = lib().lbm_cu_server_lattice(self.h, sid)
        if not h:
            raise LbmError(lib().lbm_cu_last_error().decode())
        return Lattice(c.nx, c.ny, c.nz, c.storage, self.store_velocity, False, handle=h, owner=self)

    def release(self, sid):
        check(lib().lbm_cu_server_release(self.h, sid))

    def status(self):
        q, a, used, cu = C.c_int(), C.c_int(), C.c_double(), C.c_int64()
        check(lib().lbm_cu_server_status(self.h, C.byref(q), C.byref(a), C.byref(used), C.byref(cu)))
        return {"queued": q.value, "active": a.value, "hbm_used": used.value, "cell_updates": cu.value}
