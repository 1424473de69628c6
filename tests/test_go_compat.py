"""The reference's own ctypes bridge, pointed at this library.

goSimulation/pythonBind.py:49-92 binds ``wrapperSimulate*`` with GoSlice
arguments (and an extra ``time`` double the Go signature does not have);
parrallelSimulationBind.py:50-66 binds ``parallelSimulations``.  These tests
build the same argument lists with ctypes and call this library."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu


class GoSlice(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_double)), ("len", C.c_longlong), ("cap", C.c_longlong)]


def slice_of(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return GoSlice(a.ctypes.data_as(C.POINTER(C.c_double)), a.size, a.size), a


def lib_as_go():
    return C.CDLL(os.path.join(REPO, "kmc_dn_gb300", "libkmc_dn_gb300.so"))


def _net():
    from kmc_dn_gb300 import workloads
    return workloads.plain_network(8)


@pytest.mark.parametrize("fn", ["wrapperSimulate", "wrapperSimulateRecord"])
def test_wrapper_simulate_through_reference_argtypes(engine_lib, fn):
    n = _net()
    N, P, S = n.N, n.P, n.S
    lib = lib_as_go()
    f = getattr(lib, fn)
    f.argtypes = [C.c_longlong, C.c_longlong, C.c_double, C.c_double, C.c_double, C.c_double,
                  C.c_double, GoSlice, GoSlice, GoSlice, GoSlice, GoSlice, GoSlice, C.c_int, C.c_bool,
                  GoSlice, GoSlice]
    f.restype = C.c_double
    keep = []
    sl = lambda a: (lambda s_a: (keep.append(s_a[1]), s_a[0])[1])(slice_of(a))  # noqa: E731
    occ = sl(n.occupation.astype(float))
    eo_arr = np.zeros(P)
    eo = GoSlice(eo_arr.ctypes.data_as(C.POINTER(C.c_double)), P, P)
    tr_arr = np.zeros(S * S)
    av_arr = np.zeros(N)
    tr = GoSlice(tr_arr.ctypes.data_as(C.POINTER(C.c_double)), S * S, S * S)
    av = GoSlice(av_arr.ctypes.data_as(C.POINTER(C.c_double)), N, N)
    t = f(N, P, n.nu, n.kT, n.I_0, n.R, 0.0, occ, sl(n.distances.ravel()), sl(n.E_constant()),
          sl(n.transitions_constant.ravel()), eo, sl(n.site_energies()), 20000, True, tr, av)
    assert t > 0, t
    assert eo_arr.sum() < 0                     # empty start: holes flow in
    tr = tr_arr.reshape(S, S)
    np.testing.assert_allclose(tr, -tr.T)            # net traffic: +1 from->to, -1 to->from
    # what an electrode absorbed is the net traffic into it
    np.testing.assert_allclose(eo_arr, tr[:, N:].sum(axis=0))
    assert np.all(av_arr >= 0) and np.all(av_arr <= t * (1 + 1e-9))


def test_parallel_simulations_through_reference_argtypes(engine_lib):
    import platform
    if platform.machine().lower() in ("aarch64", "arm64"):
        # ctypes' libffi on this platform does not pass fourteen 24-byte
        # structs per the C ABI (a call crashed the caller's process before
        # the callee ran); the reference's parrallelSimulationBind has the
        # same limitation there.  The export itself is exercised on x86-64.
        pytest.skip("ctypes cannot pass fourteen GoSlice structs on aarch64")
    n = _net()
    N, P, S = n.N, n.P, n.S
    nc = 6
    lib = lib_as_go()
    lib.parallelSimulations.argtypes = [GoSlice] * 14
    lib.parallelSimulations.restype = C.c_longlong
    V = np.random.default_rng(1).uniform(-1, 1, (nc, P))
    arrays = dict(
        NSites=np.full(nc, N, float), NElectrodes=np.full(nc, P, float), nu=np.full(nc, n.nu),
        kT=np.full(nc, n.kT), I_0=np.full(nc, n.I_0), R=np.full(nc, n.R),
        occupation=np.tile(n.occupation.astype(float), nc),
        distances=np.tile(n.distances.ravel(), nc), E_constant=np.concatenate([n.E_constant(v) for v in V]),
        transitions_constant=np.tile(n.transitions_constant.ravel(), nc),
        electrode_occupation=np.zeros(nc * P), hops=np.full(nc, 5000.0), time=np.zeros(nc),
        site_energies=np.concatenate([np.concatenate([np.zeros(N), v]) for v in V]))
    order = ["NSites", "NElectrodes", "nu", "kT", "I_0", "R", "occupation", "distances", "E_constant",
             "transitions_constant", "electrode_occupation", "hops", "time", "site_energies"]
    slices = [GoSlice(arrays[k].ctypes.data_as(C.POINTER(C.c_double)), arrays[k].size, arrays[k].size)
              for k in order]
    lib.kmc_goslice_abi_probe.argtypes = [GoSlice] * 14
    lib.kmc_goslice_abi_probe.restype = C.c_longlong
    want = sum((k + 1) * arrays[name].size for k, name in enumerate(order))
    got = lib.kmc_goslice_abi_probe(*slices)
    if got != want:
        import platform
        pytest.skip(f"ctypes on {platform.machine()} does not pass fourteen 24-byte structs per the "
                    f"platform C ABI (probe {got} != {want}); the reference's parrallelSimulationBind "
                    f"cannot call parallelSimulations here either")
    rc = lib.parallelSimulations(*slices)
    if rc != 0:
        buf = C.create_string_buffer(512)
        lib.kmc_last_error(buf, 512)
        raise AssertionError(f"parallelSimulations returned {rc}: {buf.value.decode()}")
    assert np.all(arrays["time"] > 0)
    eo = arrays["electrode_occupation"].reshape(nc, P)
    # hole number conservation per chain: electrodes absorb what acceptors lose
    assert np.all(np.abs(eo.sum(1)) <= N)
