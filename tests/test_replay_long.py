"""Long replays of the batched FP32 engine against the FP64 oracle.

The oracle makes a replay stream on which every hop's event uniform lies at
least 1e-4 of the total rate away from the cumulative boundaries of the pair
the FP64 loop (the reference's numba loop, kmc_dopant_networks.py:33-135)
selects; uniforms closer than that are redrawn (oracle_clear_stream).  The
FP32 engine's cumulative rates differ from the FP64 ones by far less than
1e-4 of the total, so on such a stream it must make the same hop sequence as
the FP64 loop for every hop: these tests compare the whole logs, and along
them the engine's FP32 total rate and chosen-pair rate with the oracle's
FP64 ones (the rate-level error that any current bias comes from).
"""
import functools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MARGIN = 1e-4
# Rate-level tolerances on the replay path, per network size: the FP32 total
# rate and the chosen pair's probability (its rate / total) against the FP64
# ones.  What sets them is the FP32 site energies (values of a few hundred kT
# carried by incremental updates between re-anchors: an energy error dE
# changes a rate by a relative dE/kT), so they grow with N; all stay well
# below the 1 % current criterion.
TOLERANCES = {30: dict(total=1e-4, prob=1e-3), 300: dict(total=2e-3, prob=5e-3)}


def _network(N):
    from kmc_dn_gb300 import workloads
    if N == 30:
        return workloads.plain_network(0)
    return workloads.large_network(seed=3, N=N, M=N // 10)


@functools.lru_cache(maxsize=None)
def _reference(N, hops, seed):
    import oracle as orc
    net = _network(N)
    occ = net.occupation.astype(np.uint8)
    u, redraws = orc.clear_stream(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances,
                                  net.E_constant(), net.site_energies(), net.transitions_constant, hops,
                                  seed, MARGIN)
    o = orc.numba_replay(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances, net.E_constant(),
                         net.site_energies(), net.transitions_constant, u, record=True)
    assert o["margins"].min() >= MARGIN
    return net, u, o, redraws


def _engine(net, u, hops, lanes, pair_mode):
    from kmc_dn_gb300 import _native
    from kmc_dn_gb300.engine import Batch, TableSpec
    spec = TableSpec.from_network(net) if pair_mode == "positions" else \
        TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
    b = Batch([spec], [0], [net.kT], [net.E_constant()], [net.electrodes[:, 3]],
              [net.occupation.astype(np.uint8)], [hops], replay=[u], lanes=lanes, pair_mode=pair_mode,
              record=_native.RECORD_NUMBA, hop_log=True, hop_rates=True)
    return b.run().results()


def _check(net, o, r, hops, label):
    tol = TOLERANCES[net.N]
    assert r["status"][0] == 0
    log = r["hop_log"][0]
    mism = np.flatnonzero(np.any(log != o["hop_log"], axis=1))
    assert mism.size == 0, f"{label}: first divergence at hop {mism[0]} of {hops}"
    np.testing.assert_array_equal(r["electrode_occupation"][0], o["electrode_occupation"])
    np.testing.assert_array_equal(r["occupation"][0], o["occupation"].astype(bool))
    np.testing.assert_array_equal(r["traffic"][0], o["traffic"].astype(np.int32))
    rates = r["hop_rates"][0].astype(np.float64)
    tot_err = np.abs(rates[:, 0] / o["hop_totals"] - 1.0)
    p32 = rates[:, 1] / rates[:, 0]
    p64 = o["hop_rates"] / o["hop_totals"]
    prob_err = np.abs(p32 / p64 - 1.0)
    assert tot_err.max() <= tol["total"], (label, float(tot_err.max()), float(prob_err.max()))
    assert prob_err.max() <= tol["prob"], (label, float(tot_err.max()), float(prob_err.max()))
    assert abs(r["time"][0] / o["time"] - 1.0) <= tol["total"]
    return float(tot_err.max()), float(prob_err.max())


@pytest.mark.parametrize("lanes,pair_mode", [(4, "table"), (8, "table"), (16, "table"), (32, "table"),
                                              (64, "table"), (128, "table"), (16, "positions"),
                                              (32, "positions"), (128, "positions")])
def test_engine_follows_fp64_hop_sequence_for_1e5_hops(engine_lib, lanes, pair_mode):
    """N = 30, P = 8 (the homogeneous workload's network): 10^5 hops, every
    hop identical to the FP64 loop's, for every lane width and both pair
    modes; final state, electrode counts and traffic equal; FP32 total and
    chosen-pair probability within the rate-level tolerances on every hop."""
    hops = 100_000
    net, u, o, _ = _reference(30, hops, 77)
    r = _engine(net, u, hops, lanes, pair_mode)
    _check(net, o, r, hops, f"N=30 G={lanes} {pair_mode}")


@pytest.mark.parametrize("lanes,pair_mode", [(32, "table"), (128, "table"), (128, "positions"),
                                              (256, "positions")])
def test_engine_follows_fp64_hop_sequence_large_network(engine_lib, lanes, pair_mode):
    """N = 300, P = 8 (multi-word occupancy bitmask, block groups): 2*10^4
    hops identical to the FP64 loop's (the oracle's dense FP64 loop costs
    S^2 exponentials per hop, so this case is shorter)."""
    hops = 20_000
    net, u, o, _ = _reference(300, hops, 78)
    r = _engine(net, u, hops, lanes, pair_mode)
    _check(net, o, r, hops, f"N=300 G={lanes} {pair_mode}")


def _uneven_cases():
    """Three networks of the uneven workload's distributions with temperatures
    and localisation lengths far from 1 (kT 0.5..5, ab/R 0.5..2) and 4 to 12
    electrodes."""
    from kmc_dn_gb300 import workloads
    nets = [n for n, _ in workloads.uneven_batch(64, seed=123, hops_range=(1000, 1000))]
    lo = min(nets, key=lambda n: n.kT)
    hi = max(nets, key=lambda n: n.kT)
    wide = max(nets, key=lambda n: n.ab / n.R)
    return [lo, hi, wide]


@functools.lru_cache(maxsize=None)
def _uneven_reference(k, hops, seed):
    import oracle as orc
    net = _uneven_cases()[k]
    occ = net.occupation.astype(np.uint8)
    u, _ = orc.clear_stream(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances, net.E_constant(),
                            net.site_energies(), net.transitions_constant, hops, seed, MARGIN)
    o = orc.numba_replay(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances, net.E_constant(),
                         net.site_energies(), net.transitions_constant, u, record=True)
    return net, u, o


@pytest.mark.parametrize("k", [0, 1, 2], ids=["coldest", "hottest", "widest_ab"])
@pytest.mark.parametrize("pair_mode", ["table", "positions"])
def test_engine_follows_fp64_on_uneven_networks(engine_lib, k, pair_mode):
    """Networks with kT from 0.5 to 5 and ab/R from 0.5 to 2: 10^4 hops of a
    boundary-clear stream identical to the FP64 loop's, at the default lanes
    for their size, in both pair modes."""
    from kmc_dn_gb300.engine import default_lanes
    hops = 10_000
    net, u, o = _uneven_reference(k, hops, 90 + k)
    r = _engine(net, u, hops, default_lanes(net.S), pair_mode)
    assert r["status"][0] == 0
    mism = np.flatnonzero(np.any(r["hop_log"][0] != o["hop_log"], axis=1))
    assert mism.size == 0, f"N={net.N} kT={net.kT:.2f}: first divergence at hop {mism[0]}"
    np.testing.assert_array_equal(r["electrode_occupation"][0], o["electrode_occupation"])
    np.testing.assert_array_equal(r["occupation"][0], o["occupation"].astype(bool))
    rates = r["hop_rates"][0].astype(np.float64)
    p32 = rates[:, 1] / rates[:, 0]
    p64 = o["hop_rates"] / o["hop_totals"]
    assert np.max(np.abs(rates[:, 0] / o["hop_totals"] - 1.0)) <= 2e-3
    assert np.max(np.abs(p32 / p64 - 1.0)) <= 5e-3
