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


PRUNE_CUT = 1e-2     # drops 58 % of this network's pairs, the far ones


def _pruned_mask(n, cut):
    from kmc_dn_gb300.engine import prune
    return prune(n.transitions_constant, cut) == 0.0


def test_wrapper_simulate_pruned_through_reference_argtypes(engine_lib, oracle_mod):
    """wrapperSimulatePruned (simulation.go:199-215, simulationWrapper.go:
    98-110) called with pythonBind's argtypes for it (the cut as the third
    argument): no traffic on any pair the cut removes, net traffic
    antisymmetric, and the electrode currents of repeated calls within 3
    sigma of the oracle's restatement of the Go loop run on the same pruned
    constants (both start empty, both run the same hop budget)."""
    n = _net()
    N, P, S = n.N, n.P, n.S
    lib = lib_as_go()
    f = lib.wrapperSimulatePruned
    f.argtypes = [C.c_longlong, C.c_longlong, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                  C.c_double, GoSlice, GoSlice, GoSlice, GoSlice, GoSlice, GoSlice, C.c_int, C.c_bool,
                  GoSlice, GoSlice]
    f.restype = C.c_double
    pruned = _pruned_mask(n, PRUNE_CUT)
    hops, calls, reps = 20000, 24, 48
    keep = []
    sl = lambda a: (lambda s_a: (keep.append(s_a[1]), s_a[0])[1])(slice_of(a))  # noqa: E731
    cur = []
    for _ in range(calls):
        eo_arr, tr_arr, av_arr = np.zeros(P), np.zeros(S * S), np.zeros(N)
        eo = GoSlice(eo_arr.ctypes.data_as(C.POINTER(C.c_double)), P, P)
        tr = GoSlice(tr_arr.ctypes.data_as(C.POINTER(C.c_double)), S * S, S * S)
        av = GoSlice(av_arr.ctypes.data_as(C.POINTER(C.c_double)), N, N)
        t = f(N, P, PRUNE_CUT, n.nu, n.kT, n.I_0, n.R, 0.0, sl(n.occupation.astype(float)),
              sl(n.distances.ravel()), sl(n.E_constant()), sl(n.transitions_constant.ravel()), eo,
              sl(n.site_energies()), hops, True, tr, av)
        assert t > 0, t
        traffic = tr_arr.reshape(S, S)
        assert np.all(traffic[pruned] == 0), "a pruned pair carried traffic"
        np.testing.assert_allclose(traffic, -traffic.T)
        np.testing.assert_allclose(eo_arr, traffic[:, N:].sum(axis=0))
        cur.append(eo_arr / t)
    cur = np.array(cur)
    from kmc_dn_gb300.engine import prune
    tcp = prune(n.transitions_constant, PRUNE_CUT)
    ref = []
    for s in range(reps):
        o = oracle_mod.go_simulate(N, P, n.nu, n.kT, n.I_0, n.R, np.zeros(N, np.uint8), n.distances,
                                   n.E_constant(), n.site_energies(), tcp, hops, seed=700 + s, record=True)
        assert np.all(o["traffic"][pruned] == 0)
        ref.append(o["electrode_occupation"] / o["time"])
    ref = np.array(ref)
    se = np.sqrt(cur.var(0, ddof=1) / calls + ref.var(0, ddof=1) / reps)
    z = np.abs(cur.mean(0) - ref.mean(0)) / np.maximum(se, 1e-300)
    assert np.all(z < 3.5), z


def test_go_simulation_pruned_matches_oracle(engine_lib, oracle_mod):
    """kmc_dn.go_simulation(goSpecificFunction="wrapperSimulatePruned",
    prune_threshold=cut) on the FP32 engine: no traffic on pruned pairs, and
    the currents of many such runs (the same code path, batched) within 3
    sigma of the oracle's Go loop on the same pruned constants."""
    from kmc_dn_gb300 import _native
    from kmc_dn_gb300.engine import Batch, TableSpec, prune
    from kmc_dn_gb300.kmc_dn import kmc_dn
    n = _net()
    N, P = n.N, n.P
    pruned = _pruned_mask(n, PRUNE_CUT)
    dn = kmc_dn(N, n.M, n.xdim, n.ydim, 0, electrodes=n.electrodes, acceptors=n.acceptors,
                donors=n.donors, I_0=n.I_0 / n.kT, a=n.ab / n.R)
    np.testing.assert_array_equal(dn.distances, n.distances)
    dn.go_simulation(hops=20000, goSpecificFunction="wrapperSimulatePruned", prune_threshold=PRUNE_CUT,
                     record=True, seed=5)
    assert np.all(np.asarray(dn.traffic)[pruned] == 0)
    hops, reps_gpu, reps_cpu = 20000, 256, 48
    tcp = prune(n.transitions_constant, PRUNE_CUT)
    spec = TableSpec(N, P, n.nu, n.I_0, n.R, n.distances, tcp)
    b = Batch([spec], [0] * reps_gpu, [n.kT] * reps_gpu, [n.E_constant()] * reps_gpu,
              [n.electrodes[:, 3]] * reps_gpu, [np.zeros(N, np.uint8)] * reps_gpu, [hops] * reps_gpu,
              seed=31, record=_native.RECORD_GO)
    r = b.run().results()
    assert np.all(r["status"] == 0)
    assert all(np.all(t[pruned] == 0) for t in r["traffic"])
    cur = np.array([e / t for e, t in zip(r["electrode_occupation"], r["time"])])
    ref = np.array([(lambda o: o["electrode_occupation"] / o["time"])(
        oracle_mod.go_simulate(N, P, n.nu, n.kT, n.I_0, n.R, np.zeros(N, np.uint8), n.distances,
                               n.E_constant(), n.site_energies(), tcp, hops, seed=900 + s))
        for s in range(reps_cpu)])
    se = np.sqrt(cur.var(0, ddof=1) / reps_gpu + ref.var(0, ddof=1) / reps_cpu)
    z = np.abs(cur.mean(0) - ref.mean(0)) / np.maximum(se, 1e-300)
    assert np.all(z < 3.5), z
