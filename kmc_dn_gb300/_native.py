"""ctypes binding of the engine's C ABI (include/kmc_dn_gb300.h).

The shared library is built in-tree by ``kmc_dn_gb300.build``.  There is no
fallback: if the library is missing or cannot be loaded, every entry point
raises ``NativeLibraryError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

__all__ = ["lib", "check", "KmcError", "NativeLibraryError", "KmcBatch", "LIB_PATH",
           "KMC_OK", "KMC_ERR_INVALID", "KMC_ERR_CUDA", "KMC_ERR_OOM", "KMC_ERR_TIMEOUT",
           "KMC_ERR_NONFINITE", "KMC_ERR_CANCELLED", "RECORD_NONE", "RECORD_NUMBA", "RECORD_GO",
           "PAIRS_TABLE", "PAIRS_POSITIONS",
           "EXPORTED", "KmcMfBatch", "KmcF64Batch", "MF_RATES_F64", "MF_RATES_F32"]

HERE = os.path.dirname(os.path.abspath(__file__))
# KMC_DN_GB300_LIB selects another build of the same ABI (the debug-checks or
# section-clocks library of kmc_dn_gb300/build.py)
LIB_PATH = os.environ.get("KMC_DN_GB300_LIB", os.path.join(HERE, "libkmc_dn_gb300.so"))

KMC_OK = 0
KMC_ERR_INVALID = -1
KMC_ERR_CUDA = -2
KMC_ERR_OOM = -3
KMC_ERR_TIMEOUT = -4
KMC_ERR_NONFINITE = -5
KMC_ERR_CANCELLED = -6
RECORD_NONE, RECORD_NUMBA, RECORD_GO = 0, 1, 2
PAIRS_TABLE, PAIRS_POSITIONS = 0, 1
MF_RATES_F64, MF_RATES_F32 = 0, 1

_vp = C.c_void_p
_i32, _i64, _u64, _f64, _sz = C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_size_t


class KmcError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"kmc error {code}: {message}")
        self.code = code


class NativeLibraryError(RuntimeError):
    pass


class KmcBatch(C.Structure):
    """Mirror of ``struct kmc_batch`` (all pointers are device addresses)."""
    _fields_ = [
        ("n_tables", _i32), ("max_sites", _i32),
        ("tab_N", _vp), ("tab_P", _vp), ("tab_off", _vp), ("tab_LB", _vp),
        ("n_chains", _i32), ("lanes_per_chain", _i32),
        ("chain_tab", _vp), ("chain_kT", _vp), ("chain_site_off", _vp), ("chain_el_off", _vp),
        ("chain_pair_off", _vp), ("E_constant", _vp), ("el_energy", _vp), ("occupation", _vp),
        ("electrode_occupation", _vp), ("time", _vp), ("hops_done", _vp), ("hops_total", _vp),
        ("stream", _vp), ("status", _vp), ("n_pairs", _vp), ("occ_time", _vp),
        ("occ_since", _vp), ("traffic", _vp),
        ("work", _vp), ("n_work", _i32), ("record", _i32), ("reanchor", _i32),
        ("warps_per_block", _i32), ("max_hops_per_launch", _i64), ("seed", _u64),
        ("replay", _vp), ("replay_off", _vp), ("cancel", _vp),
        ("pair_mode", _i32), ("tab_pos", _vp), ("tab_pos_off", _vp), ("tab_coef", _vp),
        ("time_budget_ns", _i64),
        ("hop_log", _vp), ("hop_rates", _vp), ("hop_log_off", _vp), ("select_mismatch", _vp),
        ("energy_drift", _vp), ("work_counter", _vp), ("flux_time", _vp),
        ("max_grid", _i32), ("uniform_kT", C.c_float),
    ]


class KmcF64Batch(C.Structure):
    """Mirror of ``struct kmc_f64_batch`` (device addresses)."""
    _fields_ = [
        ("n_chains", _i32), ("max_sites", _i32), ("record", _i32),
        ("N", _vp), ("P", _vp), ("nu", _vp), ("kT", _vp), ("I_0", _vp), ("R", _vp),
        ("pair_off", _vp), ("distances", _vp), ("transitions_constant", _vp),
        ("site_off", _vp), ("E_constant", _vp), ("se_off", _vp), ("site_energies", _vp),
        ("occupation", _vp), ("el_off", _vp), ("electrode_occupation", _vp), ("hops", _vp),
        ("seeds", _vp), ("traffic_off", _vp), ("traffic", _vp), ("occupations_in_time", _vp),
        ("time_out", _vp), ("status_out", _vp), ("flux_time", _vp), ("workspace", _vp),
        ("workspace_bytes", _sz),
    ]


class KmcMfBatch(C.Structure):
    """Mirror of ``struct kmc_mf_batch`` (device addresses for kmc_mf_run,
    host addresses for kmc_mf_run_host)."""
    _fields_ = [
        ("n_chains", _i32), ("max_sites", _i32), ("rates", _i32), ("record", _i32),
        ("N", _vp), ("P", _vp), ("nu", _vp), ("kT", _vp), ("I_0", _vp), ("R", _vp),
        ("pair_off", _vp), ("distances", _vp), ("transitions_constant", _vp),
        ("site_off", _vp), ("E_constant", _vp), ("site_energies", _vp), ("occupation", _vp),
        ("el_off", _vp), ("electrode_occupation", _vp), ("hops", _vp),
        ("traffic_off", _vp), ("traffic", _vp), ("average_occupation", _vp),
        ("time", _vp), ("status", _vp), ("iterations_done", _vp),
    ]


# name -> (restype, argtypes); every symbol include/kmc_dn_gb300.h declares
_SIGS = {
    "kmc_version": (C.c_int, []),
    "kmc_last_error": (C.c_int, [C.c_char_p, _sz]),
    "kmc_simulate_f64_workspace_size": (_sz, [_i32]),
    "kmc_simulate_f64": (C.c_int, [_i32, _i32, _f64, _f64, _f64, _f64, _vp, _vp, _vp, _vp, _vp, _vp,
                                   _i64, _i32, _vp, _vp, _vp, _u64, _vp, _vp, _vp, _vp, _sz, _vp]),
    "kmc_simulate_f64_flux": (C.c_int, [_i32, _i32, _f64, _f64, _f64, _f64, _vp, _vp, _vp, _vp, _vp, _vp,
                                        _i64, _i32, _vp, _vp, _vp, _u64, _vp, _vp, _vp, _vp, _sz, _vp, _vp]),
    "kmc_simulate_f64_batch_workspace_size": (_sz, [_i32, _i32]),
    "kmc_simulate_f64_batch": (C.c_int, [C.POINTER(KmcF64Batch), _vp]),
    "kmc_simulate_f64_static": (C.c_int, [_i32, _i32, _f64, _f64, _f64, _f64, _vp, _vp, _vp, _vp, _vp,
                                          _vp, _i64, _i32, _vp, _vp, _vp, _u64, _vp, _vp, _vp, _vp]),
    "kmc_build_table": (C.c_int, [_i32, _i32, _f64, _f64, _f64, _vp, _vp, _vp, _vp]),
    "kmc_site_energies": (C.c_int, [_i32, _i32, _i32, _vp, _vp, _f64, _vp, _vp, _vp, _vp]),
    "kmc_run_batch": (C.c_int, [C.POINTER(KmcBatch), _vp]),
    "kmc_engine_lane_options": (C.c_int, []),
    "kmc_measure_ex2_rate": (C.c_int, [C.POINTER(_f64)]),
    "kmc_preload_kernels": (C.c_int, []),
    "kmc_section_clocks": (C.c_int, [_vp, _i32]),
    "kmc_run_batch_host": (C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _vp,
                                     _vp, _vp, _vp, _vp, _u64, _i32, _vp, _vp, _vp]),
    "kmc_cancel_word_create": (C.c_int, [_vp, _vp]),
    "kmc_cancel_word_destroy": (None, [_vp]),
    "kmc_engine_create": (C.c_int, [_vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp,
                                    _vp, _vp, _vp, _u64, _i32, _i32, _vp]),
    "kmc_engine_run": (C.c_int, [_vp, _i64]),
    "kmc_engine_read": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "kmc_engine_destroy": (None, [_vp]),
    "kmc_mf_max_sites": (_i32, [_i32]),
    "kmc_mf_smem_bytes": (_sz, [_i32, _i32]),
    "kmc_mf_run": (C.c_int, [C.POINTER(KmcMfBatch), _vp]),
    "kmc_mf_run_host": (C.c_int, [C.POINTER(KmcMfBatch), _vp]),
    "kmc_laplace_workspace_size": (_sz, [_i32, _i32, _i32]),
    "kmc_laplace_basis": (C.c_int, [_i32, _i32, _f64, _f64, _i32, _vp, _vp, _sz, _vp]),
    "kmc_p1_sample": (C.c_int, [_i32, _i32, _f64, _f64, _i32, _vp, _i32, _vp, _vp, _vp]),
}
EXPORTED = tuple(_SIGS)

_LIB = None
_LOCK = threading.Lock()


def lib():
    """Load (once) and return the engine library; raise if it is absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOCK:
        if _LIB is None:
            if not os.path.exists(LIB_PATH):
                raise NativeLibraryError(
                    f"{LIB_PATH} is missing: build it with `python -m kmc_dn_gb300.build` "
                    "(CUDA toolkit with sm_103a support required); there is no CPU fallback")
            try:
                L = C.CDLL(LIB_PATH)
            except OSError as e:
                raise NativeLibraryError(f"cannot load {LIB_PATH}: {e}") from e
            for name, (res, args) in _SIGS.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _LIB = L
    return _LIB


def last_error():
    buf = C.create_string_buffer(512)
    code = lib().kmc_last_error(buf, 512)
    return code, buf.value.decode(errors="replace")


def check(rc):
    """Raise KmcError for a non-zero status."""
    if rc != KMC_OK:
        _, msg = last_error()
        raise KmcError(rc, msg)
    return rc
