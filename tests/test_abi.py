"""The C-ABI library loads on the CPU host and exports every function that
include/kmc_dn_gb300.h declares (no compute calls: no GPU here)."""
import ctypes as C
import os
import re

import numpy as np

from conftest import REPO


def declared_functions(header=None):
    """Function names declared in include/*.h (or one header)."""
    import glob
    paths = [os.path.join(REPO, "include", header)] if header else glob.glob(os.path.join(REPO, "include", "*.h"))
    names = []
    for path in paths:
        src = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
        names += re.findall(r"^\s*(?:int|int64_t|size_t|double|void)\s+\**\s*(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "kmc_simulate_f64" in names and "kmc_run_batch" in names and "kmc_last_error" in names


def test_library_exports_every_declared_symbol(engine_lib):
    lib = C.CDLL(os.path.join(REPO, "kmc_dn_gb300", "libkmc_dn_gb300.so"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(engine_lib):
    from kmc_dn_gb300 import _native
    assert set(declared_functions("kmc_dn_gb300.h")) <= set(_native.EXPORTED)


def test_go_compat_names_exported(engine_lib):
    """The Go library's export names, so the reference's ctypes bridge can
    load this library in place of libSimulation.so."""
    names = declared_functions("kmc_goslice_compat.h")
    assert {"wrapperSimulate", "wrapperSimulateRecord", "wrapperSimulatePruned",
            "wrapperSimulateRecordPlus", "wrapperSimulateProbability", "parallelSimulations"} <= set(names)


def test_error_channel_without_gpu(engine_lib):
    """Argument validation happens before any CUDA call and reports through
    kmc_last_error."""
    from kmc_dn_gb300 import _native
    L = _native.lib()
    rc = L.kmc_build_table(-1, 0, 1.0, 1.0, 1.0, None, None, None, None)
    assert rc == _native.KMC_ERR_INVALID
    code, msg = _native.last_error()
    assert code == rc and "bad sizes" in msg
    assert L.kmc_run_batch(None, None) == _native.KMC_ERR_INVALID
    assert L.kmc_version() >= 100
    # the release library counts no section clocks (only a -DKMC_SECTION_CLOCKS build does)
    out = (C.c_uint64 * 9)()
    assert L.kmc_section_clocks(out, 0) == _native.KMC_ERR_INVALID
    assert "KMC_SECTION_CLOCKS" in _native.last_error()[1]


def _struct_fields(name):
    src = open(os.path.join(REPO, "include", "kmc_dn_gb300.h")).read()
    body = src[src.index(f"typedef struct {name} {{") + len(f"typedef struct {name} {{"):src.index(f"}} {name};")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for stmt in body.split(";"):
        if stmt.strip():
            names += [re.findall(r"\w+", d)[-1] for d in stmt.split(",")]
    return names


def test_struct_layout_matches_header():
    """ctypes mirrors of struct kmc_batch and struct kmc_mf_batch: field
    order and names as in the header."""
    from kmc_dn_gb300._native import KmcBatch, KmcMfBatch
    assert _struct_fields("kmc_batch") == [f[0] for f in KmcBatch._fields_]
    assert _struct_fields("kmc_mf_batch") == [f[0] for f in KmcMfBatch._fields_]


def test_engine_handle_rejects_bad_arguments_without_gpu(engine_lib):
    """kmc_engine_create validates its arguments before any CUDA call and
    leaves the handle NULL; run/read on a NULL handle are errors."""
    from kmc_dn_gb300._native import KMC_ERR_INVALID, last_error, lib
    L = lib()
    h = C.c_void_p()
    # n_geoms 0, eight NULL geometry arrays, n_chains 0, six NULL chain arrays,
    # seed, lanes, record, stream
    assert L.kmc_engine_create(C.byref(h), 0, *([None] * 8), 0, *([None] * 6), 0, 0, 0, None) == KMC_ERR_INVALID
    assert not h.value
    assert L.kmc_engine_run(None, 10) == KMC_ERR_INVALID
    assert "NULL engine" in last_error()[1]
    assert L.kmc_engine_read(None, None, None, None, None, None, None, None) == KMC_ERR_INVALID
    L.kmc_engine_destroy(None)          # a no-op


def test_empty_batches_are_a_no_op_without_gpu(engine_lib):
    """Zero chains: the host entry points return KMC_OK before touching the
    device (the reference's parallelSimulations returns at once too)."""
    from kmc_dn_gb300._native import KMC_OK, lib
    L = lib()
    one = np.ones(1)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    gN, gP, off = np.array([4], np.int32), np.array([2], np.int32), np.zeros(1, np.int64)
    rc = L.kmc_run_batch_host(1, p(gN), p(gP), p(one), p(one), p(one), p(off), p(np.ones(36)), p(np.ones(36)), 0,
                              None, None, None, None, None, None, 0, 0, None, None, None)
    assert rc == KMC_OK
