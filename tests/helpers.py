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


def anderson_polish(resid, x, tol=1e-13, m=8, beta=0.1, itmax=3000):
    """Drive x to the fixed point g(x) = 0 of one residual function with
    Anderson (Pulay) mixing.  The history's least-squares problem is solved
    with its columns scaled to unit norm, so it stays well conditioned down to
    the rounding floor of g.  The reference's own DIIS adds 1e-9 to every
    Gram entry (sfnewton.cpp:837-880), which leaves about one significant
    digit in that matrix once ‖Δx‖² nears 1e-24 and stalls or diverges there.
    This is test harness code: it compares the fixed points of two residual
    implementations (the device path and the oracle), not their solvers.
    Returns (x, ‖g‖₂, iterations) at the smallest residual seen."""
    X, G = [], []
    x = np.array(x, dtype=np.float64, copy=True)
    best_r, best_x, it = np.inf, x.copy(), 0
    for it in range(itmax):
        g = resid(x)
        r = float(np.linalg.norm(g))
        if not np.isfinite(r):
            break
        if r < best_r:
            best_r, best_x = r, x.copy()
        if r <= tol:
            break
        X.append(x.copy())
        G.append(g.copy())
        if len(X) > m + 1:
            X.pop(0)
            G.pop(0)
        if len(X) > 1:
            dX = np.array([X[i + 1] - X[i] for i in range(len(X) - 1)]).T
            dG = np.array([G[i + 1] - G[i] for i in range(len(G) - 1)]).T
            sc = np.linalg.norm(dG, axis=0)
            sc[sc == 0] = 1.0
            gam, *_ = np.linalg.lstsq(dG / sc, g, rcond=1e-13)
            gam = gam / sc
            x = x - beta * g - (dX - beta * dG) @ gam
        else:
            x = x - beta * g
    return best_x, best_r, it
