"""namics_gb300: GB300-native Scheutjens–Fleer SCF hot path.

The compute lives in the CUDA/C++ library ``lib/libnamics_gb300.so`` behind
the C ABI of ``include/namics_gb300.h``.  This module is a thin ctypes layer
over it for Python callers (tests, benchmarks, scripts).  There is no CPU
fallback: every compute call needs the CUDA library and a GPU, and fails
loudly without them.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import NM_FP32, NM_FP64  # noqa: F401

__all__ = ["Plan", "Context", "Batch", "Stream", "Server", "NamicsError", "load_library", "NM_FP32", "NM_FP64"]


class NamicsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"namics_gb300 error {code}: {msg}")
        self.code = code


def load_library() -> C.CDLL:
    return _abi.load()


def _check(rc: int) -> None:
    if rc != 0:
        lib = _abi.load()
        raise NamicsError(rc, lib.nm_last_error().decode(errors="replace"))


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_abi.dp)


def _check_len(x: np.ndarray, n: int, what: str) -> None:
    # the library reads and writes exactly n doubles of a host array
    if x.size != n:
        raise ValueError(f"{what}: x has {x.size} entries, the problem needs {n}")


class Plan:
    """A compiled problem: Namics input text -> lattice, segments, molecules."""

    def __init__(self, text: str):
        lib = _abi.load()
        p = _abi.P_plan()
        _check(lib.nm_plan_create(text.encode(), C.byref(p)))
        self._p = p
        self.text = text

    def __del__(self):
        try:
            if getattr(self, "_p", None):
                _abi.load().nm_plan_destroy(self._p)
                self._p = None
        except Exception:
            pass

    @property
    def ptr(self):
        return self._p

    @property
    def c(self) -> _abi.nm_plan:
        return self._p.contents

    # convenient views
    @property
    def M(self) -> int:
        return self.c.M

    @property
    def iv(self) -> int:
        return self.c.iv

    @property
    def n_seg(self) -> int:
        return self.c.n_seg

    @property
    def n_mol(self) -> int:
        return self.c.n_mol

    @property
    def seg_names(self) -> list[str]:
        return [self.c.seg_name[i].decode() for i in range(self.n_seg)]

    @property
    def it_seg(self) -> list[int]:
        return [self.c.it_seg[i] for i in range(self.c.n_it)]

    @property
    def state_names(self) -> list[str]:
        return [self.c.state_name[j].decode() for j in range(self.c.n_state)]

    @property
    def state_alphabulk(self) -> list[float]:
        return [self.c.state_alphabulk[j] for j in range(self.c.n_state)]

    def state_bulk(self, fixed_ab=None, pK=None, sp_phibulk=None):
        """The bulk equilibrium of the states (nm_plan_state_bulk): the
        states' bulk fractions and the molecules' bulk charges for the given
        fixed fractions, pK values and previous bulk volume fractions of the
        species (each None: the input's, or before any solve)."""
        c = self.c
        arr = lambda v: None if v is None else np.ascontiguousarray(v, dtype=np.float64)  # noqa: E731
        fx, pk, spb = arr(fixed_ab), arr(pK), arr(sp_phibulk)
        if fx is not None:
            _check_len(fx, c.n_state, "Plan.state_bulk fixed_ab")
        if spb is not None:
            _check_len(spb, c.n_sp, "Plan.state_bulk sp_phibulk")
        ab, q = np.empty(c.n_state), np.empty(c.n_mol)
        ptr = lambda a: _dptr(a) if a is not None else None  # noqa: E731
        _check(_abi.load().nm_plan_state_bulk(self._p, ptr(fx), ptr(pk), ptr(spb), _dptr(ab), _dptr(q)))
        return ab, q

    @property
    def it_names(self) -> list[str]:
        """Name of each iteration block's representative: the mon of an
        ItMonList block, the state of an ItStateList block (the names a
        reference guess file lists)."""
        c = self.c
        if c.n_state == 0:
            return [self.seg_names[i] for i in self.it_seg]
        names = self.seg_names + self.state_names
        return [names[c.it_sp[i]] for i in range(c.n_it)]

    @property
    def shape(self) -> tuple[int, ...]:
        c = self.c
        if c.gradients == 1:
            return (c.MX + 2,)
        if c.gradients == 2:
            return (c.MX + 2, c.MY + 2)
        return (c.MX + 2, c.MY + 2, c.MZ + 2)

    def interior_mask(self) -> np.ndarray:
        m = np.zeros(self.shape, dtype=bool)
        m[tuple(slice(1, -1) for _ in self.shape)] = True
        return m.reshape(-1)

    def scan_values(self) -> list[float]:
        """The values of the input's scan (`var : … : scan`), step 0 first;
        empty without a scan."""
        c = self.c
        if c.scan_mol < 0 and c.scan_state < 0 and c.scan_reaction < 0:
            return []
        out = []
        for k in range(c.scan_n + 1):
            v = C.c_double()
            _check(_abi.load().nm_plan_scan_value(self._p, k, C.byref(v)))
            out.append(v.value)
        return out

    def chainlength(self, mol: int) -> float:
        return self.c.mols[mol].chainlength

    def segment_updates(self) -> float:
        """Segment-site updates of one residual evaluation: 2·Σ_mol n_store·sites."""
        c = self.c
        sites = c.MX * max(c.MY, 1) * max(c.MZ, 1)
        return 2.0 * sum(c.mols[m].n_store for m in range(c.n_mol)) * sites


@dataclass
class SolveResult:
    iterations: int
    residual: float
    status: int


@dataclass
class SearchResult:
    value: float       # the searched molecule quantity at exit
    error: float       # the target's error there
    iterations: int
    solves: int
    status: int


class Context:
    """Device state for one problem (nm_ctx)."""

    def __init__(self, plan: Plan, precision: int = NM_FP64, device: int = 0, stream: int | None = None,
                 checkpoint_stride: int = 0):
        lib = _abi.load()
        self.plan = plan
        opt = _abi.nm_ctx_options(precision, checkpoint_stride, device, C.c_void_p(stream) if stream else None)
        h = C.c_void_p()
        _check(lib.nm_ctx_create(plan.ptr, C.byref(opt), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            _abi.load().nm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def residual_dev(self, x_ptr: int, g_ptr: int) -> None:
        _check(_abi.load().nm_residual_dev(self._h, C.c_void_p(x_ptr), C.c_void_p(g_ptr)))

    def solve_dev(self, x_ptr: int) -> SolveResult:
        r = _abi.nm_solve_result()
        rc = _abi.load().nm_solve_dev(self._h, C.c_void_p(x_ptr), C.byref(r))
        if rc not in (0, _abi.NM_ERR_NOT_CONVERGED) and r.status == 0:
            _check(rc)
        return SolveResult(r.iterations, r.residual, r.status if r.status else rc)

    def search(self, x_ptr: int) -> SearchResult:
        """The plan's search (`var` keys) from the device field at x_ptr,
        updated in place; the molecule's value is left at the result."""
        r = _abi.nm_search_result()
        rc = _abi.load().nm_ctx_search(self._h, C.c_void_p(x_ptr), C.byref(r))
        if rc not in (0, _abi.NM_ERR_NOT_CONVERGED):
            _check(rc)
        return SearchResult(r.value, r.error, r.iterations, r.solves, r.status)

    def solve_host(self, x: np.ndarray, want_phi: bool = True) -> tuple[SolveResult, np.ndarray | None]:
        x = np.ascontiguousarray(x, dtype=np.float64)
        _check_len(x, self.plan.iv, "Context.solve_host")
        phi = np.empty(self.plan.n_seg * self.plan.M) if want_phi else None
        r = _abi.nm_solve_result()
        rc = _abi.load().nm_solve_host(self._h, _dptr(x), _dptr(phi) if want_phi else None, C.byref(r))
        if rc not in (0, _abi.NM_ERR_NOT_CONVERGED):
            _check(rc)
        return SolveResult(r.iterations, r.residual, r.status), phi

    def field(self, which: int) -> np.ndarray:
        p = self.plan
        n = {0: p.n_seg, 1: p.n_seg, 2: 1, 3: 1, 4: p.n_mol, 5: p.n_seg, 6: 1, 7: 1, 8: 1,
             9: p.c.n_state, 10: p.c.n_state, 11: p.c.n_state}[which] * p.M
        out = np.empty(n)
        _check(_abi.load().nm_get_field(self._h, which, _dptr(out)))
        return out

    def molecule(self, m: int) -> dict:
        v = [C.c_double() for _ in range(4)]
        _check(_abi.load().nm_get_molecule(self._h, m, *[C.byref(t) for t in v]))
        return dict(GN=v[0].value, n=v[1].value, theta=v[2].value, phibulk=v[3].value)

    def free_energy(self) -> tuple[float, float, np.ndarray]:
        F, O = C.c_double(), C.c_double()
        mu = np.empty(self.plan.n_mol)
        _check(_abi.load().nm_free_energy(self._h, C.byref(F), C.byref(O), _dptr(mu)))
        return F.value, O.value, mu

    def propagate_dev(self, g_in_ptr: int, g1_ptr: int | None, g_out_ptr: int) -> None:
        _check(_abi.load().nm_propagate_dev(self._h, C.c_void_p(g_in_ptr),
                                            C.c_void_p(g1_ptr) if g1_ptr else None, C.c_void_p(g_out_ptr)))

    def side_dev(self, x_ptr: int, out_ptr: int) -> None:
        _check(_abi.load().nm_side_dev(self._h, C.c_void_p(x_ptr), C.c_void_p(out_ptr)))

    # Lattice / Molecule pieces on device arrays (pointers), see the header
    def add_phi_dev(self, phi_ptr: int, gf_ptr: int, gb_ptr: int, degeneracy: float | None = None,
                    g1_ptr: int | None = None, norm: float | None = None) -> None:
        lib, V = _abi.load(), C.c_void_p
        if g1_ptr is not None:
            _check(lib.nm_add_phi_norm_dev(self._h, V(phi_ptr), V(gf_ptr), V(gb_ptr), V(g1_ptr), float(norm)))
        elif degeneracy is not None:
            _check(lib.nm_add_phi_deg_dev(self._h, V(phi_ptr), V(gf_ptr), V(gb_ptr), float(degeneracy)))
        else:
            _check(lib.nm_add_phi_dev(self._h, V(phi_ptr), V(gf_ptr), V(gb_ptr)))

    def initiate_dev(self, g_ptr: int, gz_ptr: int) -> None:
        _check(_abi.load().nm_initiate_dev(self._h, C.c_void_p(g_ptr), C.c_void_p(gz_ptr)))

    def terminate_dev(self, gz_ptr: int, g_ptr: int) -> None:
        _check(_abi.load().nm_terminate_dev(self._h, C.c_void_p(gz_ptr), C.c_void_p(g_ptr)))

    def weighted_sum_dev(self, x_ptr: int) -> float:
        out = C.c_double()
        _check(_abi.load().nm_weighted_sum_dev(self._h, C.c_void_p(x_ptr), C.byref(out)))
        return out.value

    def compute_gn_dev(self, g_ptr: int) -> float:
        out = C.c_double()
        _check(_abi.load().nm_compute_gn_dev(self._h, C.c_void_p(g_ptr), C.byref(out)))
        return out.value

    def compose_dev(self, mol: int, x_ptr: int, rho_ptr: int) -> float:
        """Molecule::ComputePhi of molecule `mol` at the field x; returns G(N)."""
        out = C.c_double()
        _check(_abi.load().nm_compose_dev(self._h, mol, C.c_void_p(x_ptr), C.c_void_p(rho_ptr), C.byref(out)))
        return out.value

    def autotune(self, x_ptr: int) -> dict:
        """nm_ctx_autotune at the device field x: the kernel choices kept."""
        t = _abi.nm_ctx_tuning()
        _check(_abi.load().nm_ctx_autotune(self._h, C.c_void_p(x_ptr), C.byref(t)))
        return {"rows": t.rows, "tile": t.tile, "checkpoint_stride": t.checkpoint_stride, "sweep2d": t.sweep2d,
                "cluster3d": t.cluster3d, "candidates": t.candidates, "ms_per_residual": t.ms_per_residual}

    def launch_count(self) -> int:
        return int(_abi.load().nm_ctx_launch_count(self._h))

    def write_pro(self, path: str, items: list[str]) -> None:
        """Profiles of the last residual in the reference's .pro layout."""
        arr = (C.c_char_p * len(items))(*[s.encode() for s in items])
        _check(_abi.load().nm_write_pro(self._h, str(path).encode(), arr, len(items)))

    def write_kal(self, path: str, items: list[str], result: SolveResult | None = None,
                  append: bool = False) -> None:
        """Scalars of the last residual (and of `result`) in the .kal layout."""
        arr = (C.c_char_p * len(items))(*[s.encode() for s in items])
        r = None
        if result is not None:
            r = _abi.nm_solve_result()
            r.iterations, r.residual, r.status = result.iterations, result.residual, result.status
        _check(_abi.load().nm_write_kal(self._h, str(path).encode(), arr, len(items),
                                        C.byref(r) if r is not None else None, int(append)))

    def set_values(self, values: dict[str, float]) -> None:
        """Change χ, a molecule's amount or a fixed state's alphabulk for the
        next solve (a scan step)."""
        items = list(values)
        arr = (C.c_char_p * len(items))(*[s.encode() for s in items])
        v = np.ascontiguousarray([float(values[k]) for k in items], dtype=np.float64)
        _check(_abi.load().nm_ctx_set_values(self._h, arr, _dptr(v), len(items)))

    def set_option(self, option: int, value: int) -> None:
        _check(_abi.load().nm_ctx_set_option(self._h, option, value))


class Batch:
    """Many independent 1-gradient problems solved in one persistent launch
    (a device-resident work loop: resident CTAs take problems from a queue)."""

    def __init__(self, plans: list[Plan], precision: int = NM_FP64, device: int = 0, stream: int | None = None):
        lib = _abi.load()
        self.plans = plans
        arr = (_abi.P_plan * len(plans))(*[p.ptr for p in plans])
        opt = _abi.nm_ctx_options(precision, 0, device, C.c_void_p(stream) if stream else None)
        h = C.c_void_p()
        _check(lib.nm_batch_create(arr, len(plans), C.byref(opt), C.byref(h)))
        self._h = h
        offs = (C.c_longlong * (len(plans) + 1))()
        _check(lib.nm_batch_offsets(h, offs))
        self.offsets = np.array(list(offs), dtype=np.int64)

    def close(self):
        if getattr(self, "_h", None):
            _abi.load().nm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def total(self) -> int:
        return int(self.offsets[-1])

    def solve_dev(self, x_ptr: int):
        n = len(self.plans)
        it = np.zeros(n, dtype=np.int32)
        res = np.zeros(n)
        st = np.zeros(n, dtype=np.int32)
        _check(_abi.load().nm_batch_solve_dev(self._h, C.c_void_p(x_ptr), it.ctypes.data_as(_abi.ip),
                                              _dptr(res), st.ctypes.data_as(_abi.ip)))
        return it, res, st

    def solve_host(self, x: np.ndarray):
        _check_len(x, self.total, "Batch.solve_host")
        n = len(self.plans)
        it = np.zeros(n, dtype=np.int32)
        res = np.zeros(n)
        st = np.zeros(n, dtype=np.int32)
        _check(_abi.load().nm_batch_solve_host(self._h, _dptr(x), it.ctypes.data_as(_abi.ip),
                                               _dptr(res), st.ctypes.data_as(_abi.ip)))
        return it, res, st

    def residual_dev(self, x_ptr: int, g_ptr: int, precision: int) -> None:
        _check(_abi.load().nm_batch_residual_dev(self._h, C.c_void_p(x_ptr), C.c_void_p(g_ptr), precision))

    def fp32_iterations(self) -> np.ndarray:
        out = np.zeros(len(self.plans), dtype=np.int32)
        _check(_abi.load().nm_batch_stats(self._h, out.ctypes.data_as(_abi.ip)))
        return out

    def times(self) -> np.ndarray:
        """Per-problem time to convergence of the last solve (seconds from the
        start of the batch's first CTA)."""
        out = np.zeros(len(self.plans))
        _check(_abi.load().nm_batch_times(self._h, _dptr(out)))
        return out

    def timings(self) -> tuple[np.ndarray, np.ndarray]:
        """Per-problem seconds of the last solve: waiting in the queue (from
        the work loop's start to the problem's start in a slot) and solving
        (from that start to convergence)."""
        q = np.zeros(len(self.plans))
        s = np.zeros(len(self.plans))
        _check(_abi.load().nm_batch_timings(self._h, _dptr(q), _dptr(s)))
        return q, s

    def autotune(self, x_ptr: int) -> dict:
        """nm_batch_autotune from the device fields x (not changed)."""
        t = _abi.nm_batch_tuning()
        _check(_abi.load().nm_batch_autotune(self._h, C.c_void_p(x_ptr), C.byref(t)))
        return {"ctas_per_sm": t.ctas_per_sm, "slots": t.slots, "candidates": t.candidates,
                "ms_per_solve": t.ms_per_solve}

    @property
    def slots(self) -> int:
        """Resident CTAs of the work loop."""
        return int(_abi.load().nm_batch_slots(self._h))

    @slots.setter
    def slots(self, k: int) -> None:
        _check(_abi.load().nm_batch_set_slots(self._h, int(k)))

    def free_energy(self):
        n = len(self.plans)
        F = np.zeros(n)
        O = np.zeros(n)
        _check(_abi.load().nm_batch_free_energy(self._h, _dptr(F), _dptr(O)))
        return F, O

    def launch_count(self) -> int:
        return int(_abi.load().nm_batch_launch_count(self._h))


class Stream:
    """Streaming work loop for 1-gradient solves (nm_stream_*): requests are
    admitted into resident CTAs as slots free up, while the loop runs."""

    def __init__(self, device: int = 0, capacity: int = 1024, max_layers: int = 512, max_segments: int = 6,
                 max_pairs: int = 6, max_molecules: int = 3, max_store: int = 520, max_blocks: int = 8,
                 max_diis: int = 10, slots: int = 0, idle_seconds: float = 0.2):
        opt = _abi.nm_stream_options(device, capacity, max_layers, max_segments, max_pairs, max_molecules,
                                     max_store, max_blocks, max_diis, slots, idle_seconds)
        h = C.c_void_p()
        _check(_abi.load().nm_stream_create(C.byref(opt), C.byref(h)))
        self._h = h

    def submit(self, plan: Plan, x: np.ndarray, precision: int = NM_FP32) -> int:
        x = np.ascontiguousarray(x, dtype=np.float64)
        _check_len(x, plan.iv, "Stream.submit")
        t = C.c_longlong()
        _check(_abi.load().nm_stream_submit(self._h, plan.ptr, _dptr(x), precision, C.byref(t)))
        return t.value

    def wait(self, ticket: int, iv: int | None = None):
        """(SolveResult, field or None, seconds from submit to the solve's end)."""
        r = _abi.nm_solve_result()
        sec = C.c_double()
        x = np.zeros(iv) if iv else None
        _check(_abi.load().nm_stream_wait(self._h, ticket, _dptr(x) if x is not None else None, C.byref(r),
                                          C.byref(sec)))
        return SolveResult(r.iterations, r.residual, r.status), x, sec.value

    @property
    def slots(self) -> int:
        return int(_abi.load().nm_stream_slots(self._h))

    def launch_count(self) -> int:
        return int(_abi.load().nm_stream_launch_count(self._h))

    def close(self):
        if getattr(self, "_h", None):
            _abi.load().nm_stream_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request server on one GPU (nm_server_*)."""

    def __init__(self, precision: int = NM_FP32, workers: int = 4, max_batch: int = 64,
                 memory_budget: int = 64 << 30, device: int = 0, stream_slots: int = 0,
                 context_sweeps: int = 0):
        """stream_slots: resident CTAs of the 1-gradient streaming loop (0: two
        per SM; -1: no loop, 1-gradient requests in batched launches).
        context_sweeps: bit mask of the 2-D/3-D request contexts' options (1
        persistent 2-D sweeps, 2 cluster sweeps of small FP32 3-D boxes, 4 the
        device-resident solve loop)."""
        lib = _abi.load()
        opt = _abi.nm_server_options(precision, device, workers, max_batch, memory_budget, stream_slots,
                                     context_sweeps)
        h = C.c_void_p()
        _check(lib.nm_server_create(C.byref(opt), C.byref(h)))
        self._h = h
        self._plans = {}

    def submit(self, plan: Plan, x: np.ndarray) -> int:
        x = np.ascontiguousarray(x, dtype=np.float64)
        _check_len(x, plan.iv, "Server.submit")
        rid = C.c_longlong()
        _check(_abi.load().nm_server_submit(self._h, plan.ptr, _dptr(x), C.byref(rid)))
        self._plans[rid.value] = plan  # kept alive until waited for
        return rid.value

    def wait(self, rid: int):
        plan = self._plans[rid]
        x = np.empty(plan.iv)
        r = _abi.nm_solve_result()
        sec = C.c_double()
        rc = _abi.load().nm_server_wait(self._h, rid, _dptr(x), C.byref(r), C.byref(sec))
        del self._plans[rid]
        _check(rc)
        return SolveResult(r.iterations, r.residual, r.status), x, sec.value

    def launch_count(self) -> int:
        return int(_abi.load().nm_server_launch_count(self._h))

    def close(self):
        if getattr(self, "_h", None):
            _abi.load().nm_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
