"""Shared helpers of the parity tests (host side only)."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def bits(a: np.ndarray) -> np.ndarray:
    """Bit pattern view, so that comparisons are exact (and -0 != +0)."""
    a = np.ascontiguousarray(a)
    return a.view({2: np.uint16, 4: np.uint32, 8: np.uint64}[a.itemsize])


def n_diff(a, b) -> int:
    return int((bits(a) != bits(b)).sum())


def state_hash(dd, vel, rho, flags, mask) -> str:
    """Same digest as tests/golden/make_golden.py:state_hash."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(dd[:, mask]).tobytes())
    h.update(np.ascontiguousarray(vel[:, mask]).tobytes())
    h.update(np.ascontiguousarray(rho[mask]).tobytes())
    h.update(np.ascontiguousarray(flags).tobytes())
    return h.hexdigest()


def golden_hashes():
    return json.loads((GOLDEN / "hashes.json").read_text())


def golden_small(storage):
    return dict(np.load(GOLDEN / f"cavity_{storage}_12x8x8.npz"))


def max_rel(a, b, floor=1e-30):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0
