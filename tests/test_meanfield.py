"""Mean-field relaxation (Go probSimulate, goSimulation/probabilitySimulation.go:
53-157): the C oracle against a plain-Python restatement and the closed-form
single-site case, then the device kernel (kmc_mf_run) against the oracle in
both rate precisions, its batching, record mode, the Go-named export and the
``go_simulation(goSpecificFunction="wrapperSimulateProbability")`` route."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import REPO


def _oracle():
    import oracle as O
    return O


def _args(net, hops, start=0.5):
    return (net.N, net.P, net.nu, net.kT, net.I_0, net.R, np.full(net.N, start), net.distances,
            net.E_constant(), net.site_energies(), net.transitions_constant, hops)


def _single_site(E0, V, tcs, kT=1.0):
    """One acceptor, len(V) electrodes at distance 1, no interaction."""
    P = len(V)
    S = 1 + P
    d = np.ones((S, S))
    np.fill_diagonal(d, 0.0)
    tc = np.zeros((S, S))
    for e in range(P):
        tc[0, 1 + e] = tc[1 + e, 0] = tcs[e]
    return dict(N=1, P=P, nu=1.0, kT=kT, I_0=0.0, R=1.0, distances=d, transitions_constant=tc,
                E_constant=np.array([E0]), site_energies=np.concatenate([[0.0], V]))


def test_oracle_matches_python_restatement():
    from kmc_dn_gb300 import workloads
    O = _oracle()
    for seed, hops in ((3, 25), (4, 7)):
        n = workloads.plain_network(seed)
        a = O.prob_simulate(*_args(n, hops), record=True)
        b = O.prob_simulate_py(*_args(n, hops), record=True)
        for k in ("time", "occupation", "electrode_occupation", "site_energies", "traffic",
                  "average_occupation"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_oracle_single_site_current_closed_form():
    """For one site the mean-field equation is the exact master equation;
    the Go loop advances the clock by 0.98 of the step it applies
    (probabilitySimulation.go:111 vs :121), so its current is the exact
    stationary current divided by 0.98."""
    O = _oracle()
    E0, V, tcs = 0.3, np.array([0.0, 1.0]), [0.5, 0.2]
    s = _single_site(E0, V, tcs)
    r = O.prob_simulate(s["N"], s["P"], 1.0, 1.0, 0.0, 1.0, [0.5], s["distances"], s["E_constant"],
                        s["site_energies"], s["transitions_constant"], 200)
    f = lambda dE: np.exp(-dE) if dE > 0 else 1.0  # noqa: E731
    gin = np.array([tcs[e] * f(E0 - V[e]) for e in range(2)])
    gout = np.array([tcs[e] * f(V[e] - E0) for e in range(2)])
    o = gin.sum() / (gin.sum() + gout.sum())
    current = o * gout - (1 - o) * gin
    np.testing.assert_allclose(r["electrode_occupation"] / r["time"], current / 0.98, rtol=1e-3)
    # charge is conserved: what left the electrodes sits on the site
    assert abs(r["electrode_occupation"].sum() + (r["occupation"][0] - 0.5)) < 1e-12


def test_oracle_first_iteration_by_hand():
    O = _oracle()
    s = _single_site(0.3, np.array([0.0, 1.0]), [0.5, 0.2])
    r = O.prob_simulate(1, 2, 1.0, 1.0, 0.0, 1.0, [0.5], s["distances"], s["E_constant"],
                        s["site_energies"], s["transitions_constant"], 1)
    t_out = np.array([0.5 * 0.5 * 1.0, 0.5 * 0.2 * np.exp(-0.7)])    # site -> electrodes
    t_in = np.array([0.5 * 0.5 * np.exp(-0.3), 0.5 * 0.2 * 1.0])      # electrodes -> site
    tot = t_out.sum() + t_in.sum()
    diff = t_in.sum() - t_out.sum()
    assert 0 <= 0.5 + diff / tot <= 1
    np.testing.assert_allclose(r["time"], 0.98 / tot, rtol=1e-15)
    np.testing.assert_allclose(r["occupation"][0], 0.5 + diff / tot, rtol=1e-15)
    np.testing.assert_allclose(r["electrode_occupation"], (t_out - t_in) / tot, rtol=1e-14)


# --------------------------------------------------------------------------
# device
# --------------------------------------------------------------------------

def _mf_net(n):
    from kmc_dn_gb300.meanfield import Network
    return Network(n.N, n.P, n.nu, n.kT, n.I_0, n.R, n.distances, n.transitions_constant,
                   n.E_constant(), n.site_energies()[n.N:])


def _nets():
    from kmc_dn_gb300 import workloads
    out = [workloads.plain_network(s) for s in (0, 1)]
    rng = np.random.Generator(np.random.PCG64(7))
    L = float(np.sqrt(60 / workloads.DENSITY))
    out.append(workloads.make_network(rng, 60, 6, L, L, workloads.edge_thirds(L),
                                      voltages=rng.uniform(-1, 1, 8), I_0=50.0, cells=60))
    return out


def _compare(gpu, ref, n, tol):
    """Relative to the scale of each quantity: probabilities to tol, the
    time to tol, each electrode's integrated charge to tol of the largest
    electrode flow."""
    np.testing.assert_allclose(gpu["time"], ref["time"], rtol=tol)
    np.testing.assert_allclose(gpu["occupation"], ref["occupation"], atol=tol, rtol=0)
    scale = max(1.0, np.abs(ref["electrode_occupation"]).max())
    np.testing.assert_allclose(gpu["electrode_occupation"], ref["electrode_occupation"], atol=tol * scale, rtol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("rates,tol", [("f64", 1e-9), ("f32", 2e-4)])
def test_device_matches_oracle(engine_lib, rates, tol):
    """FP64 rates: the oracle's arithmetic up to summation order (1e-9).
    FP32 rates (ex2.approx, about 2 ulp): 2e-4 of each quantity's scale
    after 1000 iterations."""
    from kmc_dn_gb300 import meanfield
    O = _oracle()
    nets = _nets()
    r = meanfield.run([_mf_net(n) for n in nets], 1000, rates=rates)
    assert (r["status"] == 0).all() and (r["iterations"] == 1000).all()
    for c, n in enumerate(nets):
        ref = O.prob_simulate(*_args(n, 1000))
        _compare(dict(time=r["time"][c], occupation=r["occupation"][c],
                      electrode_occupation=r["electrode_occupation"][c]), ref, n, tol)
        np.testing.assert_allclose(r["site_energies"][c], ref["site_energies"][:n.N], atol=1e3 * tol)


@pytest.mark.gpu
def test_device_batch_is_independent_of_its_mix(engine_lib):
    from kmc_dn_gb300 import meanfield
    nets = [_mf_net(n) for n in _nets()]
    alone = meanfield.run([nets[1]], 300, rates="f32")
    mixed = meanfield.run([nets[0], nets[1], nets[2], nets[1]], [300, 300, 50, 300], rates="f32")
    for c in (1, 3):
        assert mixed["time"][c] == alone["time"][0]
        np.testing.assert_array_equal(mixed["occupation"][c], alone["occupation"][0])
        np.testing.assert_array_equal(mixed["electrode_occupation"][c], alone["electrode_occupation"][0])
    assert mixed["iterations"][2] == 50


@pytest.mark.gpu
def test_device_record_matches_oracle(engine_lib):
    from kmc_dn_gb300 import meanfield
    O = _oracle()
    n = _nets()[0]
    r = meanfield.run([_mf_net(n)], 400, rates="f64", record=True)
    ref = O.prob_simulate(*_args(n, 400), record=True)
    scale = np.abs(ref["traffic"]).max()
    np.testing.assert_allclose(r["traffic"][0], ref["traffic"], atol=1e-9 * scale, rtol=0)
    np.testing.assert_allclose(r["average_occupation"][0], ref["average_occupation"], rtol=1e-9)
    tr = r["traffic"][0]
    np.testing.assert_allclose(tr, -tr.T, atol=1e-12 * scale)
    # the electrodes' integrated charge is the net traffic into them
    np.testing.assert_allclose(r["electrode_occupation"][0], tr[:, n.N:].sum(axis=0), atol=1e-9 * scale)


@pytest.mark.gpu
def test_device_reports_a_network_without_transitions(engine_lib):
    from kmc_dn_gb300 import meanfield
    from kmc_dn_gb300._native import KMC_ERR_NONFINITE
    s = _single_site(0.0, np.array([]), [])
    net = meanfield.Network(1, 0, 1.0, 1.0, 0.0, 1.0, s["distances"], s["transitions_constant"],
                            s["E_constant"], np.zeros(0))
    r = meanfield.run([net], 10)
    assert r["status"][0] == KMC_ERR_NONFINITE and r["iterations"][0] == 0


@pytest.mark.gpu
def test_wrapper_simulate_probability_through_reference_argtypes(engine_lib):
    """The Go-named export with pythonBind's argtypes: FP64, 0.5 start, in
    place outputs, returns the time."""
    from test_go_compat import GoSlice, slice_of
    O = _oracle()
    n = _nets()[0]
    N, P, S = n.N, n.P, n.S
    lib = C.CDLL(os.path.join(REPO, "kmc_dn_gb300", "libkmc_dn_gb300.so"))
    f = lib.wrapperSimulateProbability
    f.argtypes = [C.c_longlong, C.c_longlong, C.c_double, C.c_double, C.c_double, C.c_double,
                  C.c_double, GoSlice, GoSlice, GoSlice, GoSlice, GoSlice, GoSlice, C.c_int, C.c_bool,
                  GoSlice, GoSlice]
    f.restype = C.c_double
    keep = []

    def sl(a):
        s, arr = slice_of(a)
        keep.append(arr)
        return s, arr
    occ, occ_a = sl(np.zeros(N))
    eo, eo_a = sl(np.zeros(P))
    se, se_a = sl(n.site_energies())
    tr, tr_a = sl(np.zeros(S * S))
    av, av_a = sl(np.zeros(N))
    t = f(N, P, n.nu, n.kT, n.I_0, n.R, 0.0, occ, sl(n.distances.ravel())[0], sl(n.E_constant())[0],
          sl(n.transitions_constant.ravel())[0], eo, se, 500, True, tr, av)
    ref = O.prob_simulate(*_args(n, 500), record=True)
    _compare(dict(time=t, occupation=occ_a, electrode_occupation=eo_a), ref, n, 1e-9)
    np.testing.assert_allclose(av_a, ref["average_occupation"], rtol=1e-9)
    np.testing.assert_allclose(se_a[:N], ref["site_energies"][:N], atol=1e-9)


@pytest.mark.gpu
def test_go_simulation_probability_route(engine_lib):
    """kmc_dn.go_simulation(goSpecificFunction="wrapperSimulateProbability")
    as dn_search.py:49-52 calls it: the ctypes bridge's int() truncation of
    the electrode and occupation slices (pythonBind.py:85-86) included."""
    from kmc_dn_gb300.engine import simulate_go
    O = _oracle()
    n = _nets()[0]
    t, occ, eo = simulate_go(n.N, n.P, n.nu, n.kT, n.I_0, n.R, 0.0, n.occupation, n.distances,
                             n.E_constant(), n.site_energies(), n.transitions_constant,
                             hops=1000, goSpecificFunction="wrapperSimulateProbability")
    ref = O.prob_simulate(*_args(n, 1000))
    np.testing.assert_allclose(t, ref["time"], rtol=1e-9)
    assert eo.dtype.kind == "i" and occ.dtype.kind == "i"
    for got, want in ((eo, ref["electrode_occupation"]), (occ, ref["occupation"])):
        clear = np.abs(want - np.round(want)) > 1e-6     # away from a truncation edge
        np.testing.assert_array_equal(got[clear], np.trunc(want[clear]).astype(int))
