"""Shared helpers for the parity tests."""
from __future__ import annotations

import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INF64 = np.iinfo(np.int64).max
INF32 = np.iinfo(np.int32).max
BC_RTOL = 1e-9  # |a-b| <= 1e-9 * max(|b|, 1), FP64 (summation order differs)


def golden_cases() -> list[str]:
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def bc_err(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


def assert_levels(lv, ref_lv):
    """Levels equal everywhere, unreachable included (both as INT64_MAX)."""
    lv = np.asarray(lv, dtype=np.int64)
    ref_lv = np.asarray(ref_lv, dtype=np.int64)
    bad = np.argwhere(lv != ref_lv)
    assert bad.size == 0, f"{len(bad)} level mismatches, first (root,vertex)={bad[:5].tolist()}"


def assert_sigma(sg, ref_sg, ref_lv):
    reach = np.asarray(ref_lv) != INF64
    bad = np.argwhere((np.asarray(sg) != np.asarray(ref_sg)) & reach)
    assert bad.size == 0, f"{len(bad)} sigma mismatches, first (root,vertex)={bad[:5].tolist()}"


def assert_bc(bc, ref_bc, what="bc"):
    e = bc_err(bc, ref_bc)
    assert e <= BC_RTOL, f"{what}: max relative error {e:.3e} > {BC_RTOL}"


def widen_dist(d32: np.ndarray) -> np.ndarray:
    d = d32.astype(np.int64)
    d[d32 == INF32] = INF64
    return d
