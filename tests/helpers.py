"""Shared helpers for the parity tests (golden fixture handling)."""
from __future__ import annotations

import numpy as np


def pro_column(run: dict, key: str) -> np.ndarray:
    hdr = run["pro_header"]
    return np.array(run["pro"])[:, hdr.index(key)]


def interior(plan, arr: np.ndarray) -> np.ndarray:
    """Interior sites of a [.., M] array in the reference .pro row order
    (x-major, then y, then z)."""
    shape = plan.shape
    a = arr.reshape(arr.shape[:-1] + shape)
    sl = (Ellipsis,) + tuple(slice(1, -1) for _ in shape)
    return a[sl].reshape(arr.shape[:-1] + (-1,))


def rel_err(a: np.ndarray, b: np.ndarray, floor: float = 1e-300) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.maximum(np.max(np.abs(b)), floor)
    return float(np.max(np.abs(a - b)) / scale)


def newton_tolerance(run: dict) -> float:
    """The `newton : … : tolerance` the run's input text sets (1e-7 if none)."""
    for ln in run["input"].splitlines():
        parts = [t.strip() for t in ln.split(":")]
        if len(parts) == 4 and parts[0] == "newton" and parts[2] == "tolerance":
            return float(parts[3])
    return 1e-7


def charge_scale(plan, run: dict) -> float:
    """max over sites of Σ_s |valence_s|·φ_s from the run's .pro columns: the
    size of the ion densities whose near-cancelling sum is the charge q, so
    the scale q's error is measured against."""
    c = plan.c
    tot = 0.0
    for i, seg in enumerate(plan.seg_names):
        v = abs(c.seg_valence[i])
        if v:
            tot = tot + v * np.abs(pro_column(run, f"mon_{seg}_phi"))
    return float(np.max(tot))
