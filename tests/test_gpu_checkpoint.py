"""Checkpoint / restart: a run interrupted by save, a fresh lattice and a
load continues bit for bit like the uninterrupted run, for every storage
type and for both A-A slot layouts (the counter's parity); corrupt or
mismatched files are rejected."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import n_diff

pytestmark = pytest.mark.gpu


def params(api, storage, cs=0.17, tau=0.52):
    t = np.float64(tau) if storage == api.F64 else np.float32(tau)
    inv = float(1.0 / t) if storage == api.F64 else float(np.float32(1) / t)
    return api.Params.make(inv, float(t), api.les_coefficient(cs), (0.0, 0.0, 0.0), 0.08)


def cavity(api, dims, storage):
    L = api.Lattice(*dims, storage, True, True)
    L.set_params(params(api, storage))
    L.init([api.FLAG_OBSTACLE] * 6)
    nx, ny, nz = dims
    L.write(api.FIELD_FLAGS, np.full((nz - 2) * (nx - 2), api.FLAG_VELOCITY_INJECTION, np.int32),
            origin=(1, ny - 2, 1), size=(nx - 2, 1, nz - 2))
    L.perturb((0, 0, 0), dims, 77, 2e-2)
    return L


@pytest.mark.parametrize("storage", ["f32", "f64", "f16", "bf16", "c16"])
@pytest.mark.parametrize("first", [6, 7])
def test_lattice_restart_is_bit_exact(capi, tmp_path, storage, first):
    api = capi
    st = api.STORAGE_NAMES[storage]
    dims = (72, 20, 18)  # nx a multiple of 16 bytes: the staged kernels run for the 16-bit types
    A = cavity(api, dims, st)
    A.run(0, first)
    path = tmp_path / "lat.ckpt"
    A.checkpoint_save(path, first)
    A.run(first, 9)
    B = cavity(api, dims, st)
    B.run(0, 3)  # a different state, replaced by the load
    assert B.checkpoint_load(path) == first
    B.run(first, 9)
    assert n_diff(A.read(api.FIELD_DD), B.read(api.FIELD_DD)) == 0
    assert n_diff(A.read(api.FIELD_VELOCITY), B.read(api.FIELD_VELOCITY)) == 0
    assert n_diff(A.read(api.FIELD_FLAGS), B.read(api.FIELD_FLAGS)) == 0


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_domain_restart_is_bit_exact(capi, tmp_path, storage):
    api = capi
    st = api.STORAGE_NAMES[storage]
    size, nums = (64, 48, 40), (2, 2, 1)

    def domain():
        D = api.Domain(size, nums, st, True, True)
        D.set_params(params(api, st))
        D.set_halo_mode(1)
        D.reset()
        D.perturb(91, 1e-2)
        return D

    A = domain()
    A.run(5)
    path = tmp_path / "dom.ckpt"
    A.checkpoint_save(path)
    A.run(8)
    B = domain()
    B.run(2)  # a different state and counter, replaced by the load
    B.checkpoint_load(path)
    assert B.counter == 5
    B.run(8)
    assert A.counter == B.counter == 13
    for a, b in zip(A.subdomains, B.subdomains):
        assert n_diff(a.read(api.FIELD_DD), b.read(api.FIELD_DD)) == 0


def test_checkpoint_rejects_mismatch_and_corruption(capi, tmp_path):
    api = capi
    A = cavity(api, (24, 16, 12), api.F32)
    A.run(0, 3)
    path = tmp_path / "a.ckpt"
    A.checkpoint_save(path, 3)
    with pytest.raises(api.LbmError, match="does not match"):
        cavity(api, (24, 16, 14), api.F32).checkpoint_load(path)
    with pytest.raises(api.LbmError, match="does not match"):
        cavity(api, (24, 16, 12), api.F16).checkpoint_load(path)
    raw = bytearray(path.read_bytes())
    raw[len(raw) // 2] ^= 0x40
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(bytes(raw))
    with pytest.raises(api.LbmError, match="hash mismatch"):
        cavity(api, (24, 16, 12), api.F32).checkpoint_load(bad)
    short = tmp_path / "short.ckpt"
    short.write_bytes(bytes(raw[:100]))
    with pytest.raises(api.LbmError, match="truncated"):
        cavity(api, (24, 16, 12), api.F32).checkpoint_load(short)
    with pytest.raises(api.LbmError, match="bad magic"):
        D = api.Domain((32, 32, 32), (2, 1, 1), api.F32)
        D.checkpoint_load(path)
