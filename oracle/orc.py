"""ctypes binding of the CPU oracle (oracle/liborc.so) — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the parity reference of the tests and the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liborc.so"
dp = C.POINTER(C.c_double)
_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} missing: build it with namics_gb300.build.build_oracle()")
        lib = C.CDLL(str(LIB))
        lib.orc_create.restype = C.c_void_p
        lib.orc_create.argtypes = [C.c_void_p]
        lib.orc_destroy.argtypes = [C.c_void_p]
        lib.orc_residual.argtypes = [C.c_void_p, dp, dp]
        lib.orc_solve.argtypes = [C.c_void_p, dp, C.POINTER(C.c_int), dp]
        lib.orc_solve_n.argtypes = [C.c_void_p, dp, C.c_int, C.POINTER(C.c_int), dp]
        lib.orc_get_field.argtypes = [C.c_void_p, C.c_int, dp]
        lib.orc_get_molecule.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp]
        lib.orc_free_energy.argtypes = [C.c_void_p, dp, dp, dp]
        lib.orc_propagate.argtypes = [C.c_void_p, dp, dp, dp]
        lib.orc_compose.argtypes = [C.c_void_p, dp, C.c_int, dp, dp]
        lib.orc_side.argtypes = [C.c_void_p, dp, dp]
        lib.orc_set_amount.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double]
        lib.orc_set_states.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        lib.orc_get_species_phibulk.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        lib.orc_search.argtypes = [C.c_void_p, dp, dp, dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _lib = lib
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(dp)


class Oracle:
    """CPU restatement of the reference path for one nm_plan."""

    def __init__(self, plan):
        self.plan = plan  # namics_gb300.Plan (kept alive)
        self._h = C.c_void_p(load().orc_create(C.cast(plan.ptr, C.c_void_p)))

    def __del__(self):
        try:
            if self._h:
                load().orc_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def residual(self, x: np.ndarray) -> tuple[int, np.ndarray]:
        x = np.ascontiguousarray(x, dtype=np.float64)
        g = np.zeros_like(x)
        rc = load().orc_residual(self._h, _p(x), _p(g))
        return rc, g

    def solve(self, x: np.ndarray, max_iter: int | None = None):
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        it, res = C.c_int(), C.c_double()
        if max_iter is None:
            rc = load().orc_solve(self._h, _p(x), C.byref(it), C.byref(res))
        else:
            rc = load().orc_solve_n(self._h, _p(x), max_iter, C.byref(it), C.byref(res))
        return rc, x, it.value, res.value

    def set_amount(self, mol: int, what: int, value: float) -> None:
        """A molecule amount for the next solves (what: 0 θ, 1 n, 2 φ_bulk)."""
        rc = load().orc_set_amount(self._h, mol, what, value)
        if rc:
            raise RuntimeError(f"orc_set_amount rc={rc}")

    def species_phibulk(self) -> np.ndarray:
        """Bulk volume fractions of the species of the last residual."""
        out = np.zeros(self.plan.n_seg + self.plan.c.n_state)
        rc = load().orc_get_species_phibulk(self._h, _p(out))
        if rc:
            raise RuntimeError(f"orc_get_species_phibulk rc={rc}")
        return out

    def set_states(self, alphabulk) -> None:
        """The states' bulk fractions for the next solves (a scan of a fixed
        state's alphabulk; the bulk equilibrium comes from the caller)."""
        ab = np.ascontiguousarray(alphabulk, dtype=np.float64)
        rc = load().orc_set_states(self._h, _p(ab))
        if rc:
            raise RuntimeError(f"orc_set_states rc={rc}")

    def search(self, x: np.ndarray):
        """The plan's search from x: (rc, x, value, error, iterations, solves)."""
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        v, e = C.c_double(), C.c_double()
        it, ns = C.c_int(), C.c_int()
        rc = load().orc_search(self._h, _p(x), C.byref(v), C.byref(e), C.byref(it), C.byref(ns))
        return rc, x, v.value, e.value, it.value, ns.value

    def field(self, which: int) -> np.ndarray:
        p = self.plan
        rows = {0: p.n_seg, 1: p.n_seg, 2: 1, 3: 1, 4: p.n_mol, 5: p.n_seg, 6: 1, 7: 1, 8: 1}
        n = (rows[which] if which < 9 else p.c.n_state) * p.M
        out = np.zeros(n)
        rc = load().orc_get_field(self._h, which, _p(out))
        if rc:
            raise RuntimeError(f"orc_get_field rc={rc}")
        return out

    def molecule(self, m: int) -> dict:
        v = [C.c_double() for _ in range(4)]
        load().orc_get_molecule(self._h, m, *[C.byref(t) for t in v])
        return dict(GN=v[0].value, n=v[1].value, theta=v[2].value, phibulk=v[3].value)

    def free_energy(self):
        F, O = C.c_double(), C.c_double()
        mu = np.zeros(self.plan.n_mol)
        rc = load().orc_free_energy(self._h, C.byref(F), C.byref(O), _p(mu))
        if rc:
            raise RuntimeError(f"orc_free_energy rc={rc}")
        return F.value, O.value, mu

    def compose(self, x: np.ndarray, mol: int, n_molmon: int):
        """Molecule::ComputePhi of one molecule at x: (rho [n_molmon*M], GN)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        rho = np.zeros(n_molmon * self.plan.M)
        gn = C.c_double()
        rc = load().orc_compose(self._h, _p(x), mol, _p(rho), C.byref(gn))
        if rc:
            raise RuntimeError(f"orc_compose rc={rc}")
        return rho, gn.value

    def propagate(self, g_in: np.ndarray, g1: np.ndarray | None) -> np.ndarray:
        g_in = np.ascontiguousarray(g_in, dtype=np.float64).copy()
        out = np.zeros_like(g_in)
        load().orc_propagate(self._h, _p(g_in), _p(g1) if g1 is not None else None, _p(out))
        return out

    def side(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        out = np.zeros_like(x)
        load().orc_side(self._h, _p(x), _p(out))
        return out
