"""The electrodes' expected-inflow integrals (flux_time): the compensator of
each electrode's hop count, a low-variance companion estimate of the
current used by the precision comparison.  For electrode e in a state with
rates r: J_e = sum_i r(i -> e) - sum_j r(e -> j) (holes i, empty acceptors
j; the rates of kmc_dopant_networks.py:69-87), and flux_time_e = the sum
over hops of J_e(state) * (time spent in the state)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _J_per_state(net, occ):
    """J_e of one state in FP64 with the reference's rate expressions."""
    N, P, S = net.N, net.P, net.S
    d, tc = net.distances, net.transitions_constant
    se = net.site_energies()
    IR = net.I_0 * net.R
    E = np.array(se, dtype=np.float64)
    for i in range(N):
        acc = sum((1 - occ[j]) / d[i, j] for j in range(N) if j != i)
        E[i] = net.E_constant()[i] - IR * acc
    J = np.zeros(P)
    for e in range(P):
        s = N + e
        for i in range(N):
            if occ[i]:                          # hole i -> electrode e
                dE = E[s] - E[i]
                J[e] += tc[i, s] * (net.nu * np.exp(-dE / net.kT) if dE > 0 else net.nu)
            else:                               # electrode e -> empty i
                dE = E[i] - E[s]
                J[e] -= tc[s, i] * (net.nu * np.exp(-dE / net.kT) if dE > 0 else net.nu)
    return J


def test_fp64_kernel_flux_matches_a_host_recomputation(engine_lib, oracle_mod):
    """Along a replayed run the FP64 kernel's flux_time equals the sum of
    J_e(state) * hop time recomputed on the host from the hop log."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import simulate_f64
    from kmc_dn_gb300.rng import replay_uniforms
    net = workloads.plain_network(2)
    hops = 600
    u = replay_uniforms(31, 2 * hops)
    occ0 = net.occupation.astype(np.uint8)
    r = simulate_f64(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ0, net.distances, net.E_constant(),
                     net.site_energies(), net.transitions_constant, hops, uniforms=u, hop_log=True, flux=True)
    o = oracle_mod.numba_replay(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ0, net.distances,
                                net.E_constant(), net.site_energies(), net.transitions_constant, u, record=False)
    np.testing.assert_array_equal(r["hop_log"], o["hop_log"])
    occ = occ0.copy()
    F = np.zeros(net.P)
    for k, (f, t) in enumerate(o["hop_log"]):
        F += _J_per_state(net, occ) * o["hop_times"][k]
        if f < net.N:
            occ[f] = 0
        if t < net.N:
            occ[t] = 1
    np.testing.assert_allclose(r["flux_time"], F, rtol=1e-9, atol=1e-12 * np.abs(F).max())


def test_fp32_flux_follows_fp64_flux_on_a_common_replay(engine_lib, oracle_mod):
    """On a boundary-clear replay stream both hop loops make the same hops,
    so their flux integrals differ only by FP32 rates and times: within
    1e-3 of the largest one."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec, simulate_f64
    net = workloads.plain_network(0)
    hops = 20_000
    occ = net.occupation.astype(np.uint8)
    u, _ = oracle_mod.clear_stream(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances,
                                   net.E_constant(), net.site_energies(), net.transitions_constant, hops, 5, 1e-4)
    r64 = simulate_f64(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances, net.E_constant(),
                       net.site_energies(), net.transitions_constant, hops, uniforms=u, flux=True)
    for lanes in (8, 16, 128):
        spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
        b = Batch([spec], [0], [net.kT], [net.E_constant()], [net.electrodes[:, 3]], [occ], [hops],
                  replay=[u], lanes=lanes, flux=True)
        r = b.run().results()
        np.testing.assert_array_equal(r["electrode_occupation"][0], r64["electrode_occupation"])
        f32, f64 = r["flux_time"][0], r64["flux_time"]
        assert np.max(np.abs(f32 - f64)) <= 1e-3 * np.abs(f64).max(), (lanes, f32, f64)


def test_hop_count_minus_flux_has_zero_mean(engine_lib):
    """electrode_occupation - flux_time is a zero-mean martingale: over 256
    independent FP32 chains its mean per unit time is within 4 standard
    errors of zero for every electrode, and flux_time / time estimates the
    same currents as electrode_occupation / time, with a smaller spread."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    net = workloads.plain_network(0)
    n, hops = 256, 100_000
    spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
    b = Batch([spec], [0] * n, [net.kT] * n, [net.E_constant()] * n, [net.electrodes[:, 3]] * n,
              [net.occupation.astype(np.uint8)] * n, [hops] * n, seed=71, flux=True)
    r = b.run().results()
    assert np.all(r["status"] == 0)
    T = r["time"][:, None]
    cnt = np.array(r["electrode_occupation"]) / T
    fl = np.array(r["flux_time"]) / T
    d = cnt - fl
    z = np.abs(d.mean(0)) / (d.std(0, ddof=1) / np.sqrt(n))
    assert np.all(z < 4.0), z
    assert np.median(fl.std(0) / np.maximum(cnt.std(0), 1e-300)) < 1.0
