"""ctypes mirror of include/namics_gb300.h (plain C structs and entry points)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libnamics_gb300.so"

NM_OK = 0
NM_ERR_GN = -1
NM_ERR_NAN_DIIS = -2
NM_ERR_NAN_SVD = -3
NM_ERR_NEG_SOLVENT = -4
NM_ERR_INPUT = -10
NM_ERR_CUDA = -11
NM_ERR_ARG = -12
NM_ERR_NOMEM = -13
NM_ERR_NOT_CONVERGED = -14
NM_ERR_TIMEOUT = -15
NM_OPT_SWEEP2D = 1
NM_OPT_ROWS3D = 2
NM_OPT_CHECKPOINT = 3
NM_OPT_TILE3D = 4
NM_OPT_CLUSTER3D = 5
NM_OPT_DEVICE_LOOP = 6

NM_FP64, NM_FP32 = 0, 1

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


class nm_block(C.Structure):
    _fields_ = [("seg", C.c_int), ("molmon", C.c_int), ("length", C.c_int), ("s0", C.c_int),
                ("parent", C.c_int), ("mult", C.c_int), ("degeneracy", C.c_double),
                ("n_child", C.c_int), ("child0", C.c_int)]


class nm_molecule(C.Structure):
    _fields_ = [("freedom", C.c_int), ("pinned", C.c_int), ("n", C.c_double), ("theta", C.c_double),
                ("phibulk", C.c_double), ("chainlength", C.c_double), ("n_molmon", C.c_int),
                ("molmon_seg", ip), ("molmon_fraction", dp), ("n_blocks", C.c_int),
                ("blocks", C.POINTER(nm_block)), ("child_index", ip), ("n_store", C.c_int),
                ("charge", C.c_double), ("markov", C.c_int), ("bend", C.c_double * 3)]


class nm_plan(C.Structure):
    _fields_ = [("gradients", C.c_int), ("MX", C.c_int), ("MY", C.c_int), ("MZ", C.c_int),
                ("geometry", C.c_int), ("lattice_type", C.c_int), ("stencil_full", C.c_int),
                ("bc", C.c_int * 6), ("JX", C.c_int), ("JY", C.c_int), ("M", C.c_int),
                ("lambda_", C.c_double), ("offset_first_layer", C.c_double),
                ("bond_length", C.c_double), ("volume", C.c_double),
                ("L", dp), ("lambda_1", dp), ("lambda0", dp), ("lambda1", dp), ("ksam", ip),
                ("n_seg", C.c_int), ("seg_name", C.POINTER(C.c_char_p)), ("seg_freedom", ip),
                ("seg_it", ip), ("seg_gmask", dp), ("seg_phi_frozen", dp), ("chi", dp),
                ("seg_valence", dp), ("seg_epsilon", dp), ("n_it", C.c_int), ("it_seg", ip),
                ("iv", C.c_int), ("charged", C.c_int), ("n_mol", C.c_int),
                ("mols", C.POINTER(nm_molecule)), ("solvent", C.c_int), ("neutralizer", C.c_int),
                ("diis_m", C.c_int), ("iterationlimit", C.c_int), ("max_norm", C.c_int),
                ("tolerance", C.c_double), ("deltamax", C.c_double), ("mol_name", C.POINTER(C.c_char_p)),
                ("search_mol", C.c_int), ("search_what", C.c_int), ("target_kind", C.c_int),
                ("target_mol", C.c_int), ("target_what", C.c_int), ("target_value", C.c_double),
                ("super_tolerance", C.c_double), ("super_deltamax", C.c_double),
                ("super_iterationlimit", C.c_int),
                ("scan_mol", C.c_int), ("scan_what", C.c_int), ("scan_n", C.c_int),
                ("scan_exponential", C.c_int), ("scan_start", C.c_double), ("scan_end", C.c_double),
                ("scan_step", C.c_double),
                ("save_memory", C.c_int),
                ("n_state", C.c_int), ("state_name", C.POINTER(C.c_char_p)), ("state_seg", ip),
                ("state_valence", dp), ("state_alphabulk", dp), ("state_it", ip), ("seg_nstate", ip),
                ("n_sp", C.c_int), ("chi_sp", dp), ("it_sp", ip), ("scan_state", C.c_int),
                ("scan_reaction", C.c_int)]


class nm_ctx_options(C.Structure):
    _fields_ = [("precision", C.c_int), ("checkpoint_stride", C.c_int), ("device", C.c_int),
                ("stream", C.c_void_p)]


class nm_solve_result(C.Structure):
    _fields_ = [("iterations", C.c_int), ("residual", C.c_double), ("status", C.c_int)]


class nm_search_result(C.Structure):
    _fields_ = [("value", C.c_double), ("error", C.c_double), ("iterations", C.c_int),
                ("solves", C.c_int), ("status", C.c_int)]


P_plan = C.POINTER(nm_plan)


class nm_ctx_tuning(C.Structure):
    _fields_ = [("rows", C.c_int), ("tile", C.c_int), ("checkpoint_stride", C.c_int), ("sweep2d", C.c_int),
                ("cluster3d", C.c_int), ("candidates", C.c_int), ("ms_per_residual", C.c_double)]


class nm_batch_tuning(C.Structure):
    _fields_ = [("ctas_per_sm", C.c_int), ("slots", C.c_int), ("candidates", C.c_int), ("ms_per_solve", C.c_double)]


class nm_stream_options(C.Structure):
    _fields_ = [("device", C.c_int), ("capacity", C.c_int), ("max_layers", C.c_int), ("max_segments", C.c_int),
                ("max_pairs", C.c_int), ("max_molecules", C.c_int), ("max_store", C.c_int),
                ("max_blocks", C.c_int), ("max_diis", C.c_int), ("slots", C.c_int), ("idle_seconds", C.c_double)]


class nm_server_options(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("workers", C.c_int),
                ("max_batch", C.c_int), ("memory_budget", C.c_size_t), ("stream_slots", C.c_int),
                ("context_sweeps", C.c_int)]

# (name, restype, argtypes) for every entry point declared in the header
SIGNATURES = [
    ("nm_plan_create", C.c_int, [C.c_char_p, C.POINTER(P_plan)]),
    ("nm_plan_destroy", None, [P_plan]),
    ("nm_last_error", C.c_char_p, []),
    ("nm_version", C.c_char_p, []),
    ("nm_ctx_create", C.c_int, [P_plan, C.POINTER(nm_ctx_options), C.POINTER(C.c_void_p)]),
    ("nm_ctx_destroy", C.c_int, [C.c_void_p]),
    ("nm_ctx_set_option", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("nm_ctx_set_values", C.c_int, [C.c_void_p, C.POINTER(C.c_char_p), dp, C.c_int]),
    ("nm_residual_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nm_solve_dev", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(nm_solve_result)]),
    ("nm_ctx_search", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(nm_search_result)]),
    ("nm_plan_scan_value", C.c_int, [P_plan, C.c_int, dp]),
    ("nm_plan_state_bulk", C.c_int, [P_plan, dp, dp, dp, dp, dp]),
    ("nm_solve_host", C.c_int, [C.c_void_p, dp, dp, C.POINTER(nm_solve_result)]),
    ("nm_get_field", C.c_int, [C.c_void_p, C.c_int, dp]),
    ("nm_get_molecule", C.c_int, [C.c_void_p, C.c_int, dp, dp, dp, dp]),
    ("nm_free_energy", C.c_int, [C.c_void_p, dp, dp, dp]),
    ("nm_write_pro", C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_char_p), C.c_int]),
    ("nm_write_kal", C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_char_p), C.c_int,
                               C.POINTER(nm_solve_result), C.c_int]),
    ("nm_propagate_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nm_side_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nm_add_phi_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nm_add_phi_deg_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    ("nm_add_phi_norm_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    ("nm_initiate_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nm_terminate_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nm_weighted_sum_dev", C.c_int, [C.c_void_p, C.c_void_p, dp]),
    ("nm_compute_gn_dev", C.c_int, [C.c_void_p, C.c_void_p, dp]),
    ("nm_compose_dev", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, dp]),
    ("nm_ctx_launch_count", C.c_longlong, [C.c_void_p]),
    ("nm_batch_create", C.c_int, [C.POINTER(P_plan), C.c_int, C.POINTER(nm_ctx_options), C.POINTER(C.c_void_p)]),
    ("nm_batch_destroy", C.c_int, [C.c_void_p]),
    ("nm_batch_solve_dev", C.c_int, [C.c_void_p, C.c_void_p, ip, dp, ip]),
    ("nm_batch_solve_host", C.c_int, [C.c_void_p, dp, ip, dp, ip]),
    ("nm_batch_offsets", C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    ("nm_batch_residual_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    ("nm_batch_stats", C.c_int, [C.c_void_p, ip]),
    ("nm_batch_times", C.c_int, [C.c_void_p, dp]),
    ("nm_batch_timings", C.c_int, [C.c_void_p, dp, dp]),
    ("nm_batch_slots", C.c_int, [C.c_void_p]),
    ("nm_batch_autotune", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(nm_batch_tuning)]),
    ("nm_ctx_autotune", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(nm_ctx_tuning)]),
    ("nm_batch_set_slots", C.c_int, [C.c_void_p, C.c_int]),
    ("nm_batch_free_energy", C.c_int, [C.c_void_p, dp, dp]),
    ("nm_batch_launch_count", C.c_longlong, [C.c_void_p]),
    ("nm_stream_create", C.c_int, [C.POINTER(nm_stream_options), C.POINTER(C.c_void_p)]),
    ("nm_stream_submit", C.c_int, [C.c_void_p, P_plan, dp, C.c_int, C.POINTER(C.c_longlong)]),
    ("nm_stream_wait", C.c_int, [C.c_void_p, C.c_longlong, dp, C.POINTER(nm_solve_result), C.POINTER(C.c_double)]),
    ("nm_stream_slots", C.c_int, [C.c_void_p]),
    ("nm_stream_launch_count", C.c_longlong, [C.c_void_p]),
    ("nm_stream_destroy", C.c_int, [C.c_void_p]),
    ("nm_server_create", C.c_int, [C.POINTER(nm_server_options), C.POINTER(C.c_void_p)]),
    ("nm_server_submit", C.c_int, [C.c_void_p, P_plan, dp, C.POINTER(C.c_longlong)]),
    ("nm_server_wait", C.c_int, [C.c_void_p, C.c_longlong, dp, C.POINTER(nm_solve_result), C.POINTER(C.c_double)]),
    ("nm_server_launch_count", C.c_longlong, [C.c_void_p]),
    ("nm_server_destroy", C.c_int, [C.c_void_p]),
    ("nm_solve1d_noalloc", C.c_int, [P_plan, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(nm_solve_result)]),
]

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load the product library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path or LIB_PATH)
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run namics_gb300.build.build() first")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name, None)
        if fn is None:
            continue  # reported by exported_symbols(); calling it raises
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def declared_symbols() -> list[str]:
    return [s[0] for s in SIGNATURES]


def exported_symbols() -> list[str]:
    """Declared entry points that the loaded library actually exports."""
    lib = load()
    return [n for n in declared_symbols() if getattr(lib, n, None) is not None]
