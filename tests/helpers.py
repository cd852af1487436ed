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
