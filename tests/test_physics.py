"""Known-answer physics checks (the reference's validation/ experiments):

* Boltzmann statistics: in a closed network (no electrodes) and in an open
  one at zero bias, time-averaged site occupations equal the averages over
  the exact equilibrium distribution p(s) ~ exp(-H(s)/kT), with
  H = I_0 R sum_{i<j empty} 1/d_ij - sum_{i empty} E_const_i (the Hamiltonian
  of kmc_dopant_networks.py:982-1001 with the donor term included; detailed
  balance of the Miller-Abrahams rates makes it stationary).  Restates
  validation/boltzmann_validation.py:12-64 per site instead of per state.
* Single-acceptor transistor (validation/set/set.py): the current through one
  acceptor between two electrodes equals the two-state Markov-chain value.

Averages use the correct pre-hop occupancy credit (the Go convention).
"""
import itertools

import numpy as np
import pytest

from kmc_dn_gb300 import geometry as geo

pytestmark = pytest.mark.gpu


def exact_site_occupation(Ec, d, I0R, kT, N, n_holes=None):
    states = []
    if n_holes is None:
        it = itertools.product([0, 1], repeat=N)
    else:
        it = (tuple(1 if i in c else 0 for i in range(N)) for c in itertools.combinations(range(N), n_holes))
    Hs, occs = [], []
    iu = np.triu_indices(N, 1)
    inv = 1.0 / d[:N, :N][iu]
    for s in it:
        occ = np.array(s, bool)
        empty = ~occ
        H = I0R * np.sum(inv[empty[iu[0]] & empty[iu[1]]]) - np.sum(Ec[empty])
        Hs.append(H)
        occs.append(occ)
    Hs = np.array(Hs)
    w = np.exp(-(Hs - Hs.min()) / kT)
    w /= w.sum()
    return (w[:, None] * np.array(occs)).sum(0)


def _run_record(spec, Ec, V_el, occ0, kT, chains, hops, seed):
    from kmc_dn_gb300 import _native
    from kmc_dn_gb300.engine import Batch
    b = Batch([spec], [0] * chains, [kT] * chains, [Ec] * chains, [V_el] * chains, [occ0] * chains,
              [hops] * chains, seed=seed, record=_native.RECORD_GO, lanes=8)
    r = b.run().results()
    assert np.all(r["status"] == 0)
    return np.array([o / t for o, t in zip(r["occ_time"], r["time"])]), r


def test_boltzmann_closed_network(engine_lib):
    from kmc_dn_gb300.engine import TableSpec
    rng = np.random.Generator(np.random.PCG64(3))
    N = 8
    acc, _ = geo.place_dopants(rng, N, 0, 1.0, 1.0, 0.0)
    R, _ = geo.dimensionless_R(N, 1.0, 1.0, 0.0)
    I_0, kT = 1.0, 1.0
    d = geo.site_distances(acc, np.zeros((0, 4)))
    tc = geo.transitions_constant(d, 1.0, R)
    Ec = rng.uniform(-1.5, 1.5, N)
    occ0 = np.zeros(N, np.uint8); occ0[:4] = 1
    spec = TableSpec(N, 0, 1.0, I_0, R, d, tc)
    avg, r = _run_record(spec, Ec, np.zeros(0), occ0, kT, 128, 100_000, 5)
    assert np.all([o.sum() == 4 for o in r["occupation"]])          # closed: holes conserved
    exact = exact_site_occupation(Ec, d, I_0 * R, kT, N, n_holes=4)
    m, se = avg.mean(0), avg.std(0, ddof=1) / np.sqrt(avg.shape[0])
    z = np.abs(m - exact) / (se + 1e-12)
    assert np.all(z < 3.5), (z, m, exact)


def test_boltzmann_zero_bias_open_network(engine_lib):
    from kmc_dn_gb300.engine import TableSpec
    rng = np.random.Generator(np.random.PCG64(4))
    N, P = 10, 2
    acc, _ = geo.place_dopants(rng, N, 0, 1.0, 1.0, 0.0)
    el = np.array([[0.0, 0.5, 0, 0.0], [1.0, 0.5, 0, 0.0]])       # grounded electrodes
    R, _ = geo.dimensionless_R(N, 1.0, 1.0, 0.0)
    I_0, kT = 2.0, 1.0
    d = geo.site_distances(acc, el)
    tc = geo.transitions_constant(d, 1.0, R)
    Ec = rng.uniform(-2.0, 2.0, N)
    spec = TableSpec(N, P, 1.0, I_0, R, d, tc)
    avg, r = _run_record(spec, Ec, np.zeros(P), np.zeros(N, np.uint8), kT, 128, 100_000, 6)
    exact = exact_site_occupation(Ec, d, I_0 * R, kT, N)
    m, se = avg.mean(0), avg.std(0, ddof=1) / np.sqrt(avg.shape[0])
    z = np.abs(m - exact) / (se + 1e-12)
    assert np.all(z < 3.5), (z, m, exact)


@pytest.mark.parametrize("V_S,U_G", [(1.0, 0.5), (3.0, 0.2), (-2.0, 0.0), (0.3, 1.5)])
def test_single_acceptor_transistor_current(engine_lib, V_S, U_G):
    from kmc_dn_gb300.engine import Batch, TableSpec
    acc = np.array([[0.5, 0.0, 0.0]])
    el = np.array([[0.0, 0, 0, V_S], [1.0, 0, 0, 0.0]])
    d = geo.site_distances(acc, el)
    nu, kT = 1.0, 1.0
    tc = geo.transitions_constant(d, nu, 1e5)       # ab >> R: distance does not matter
    spec = TableSpec(1, 2, nu, 1.0, 1.0, d, tc)
    chains, hops = 64, 200_000
    b = Batch([spec], [0] * chains, [kT] * chains, [[U_G]] * chains, [[V_S, 0.0]] * chains,
              [[0]] * chains, [hops] * chains, seed=9, lanes=4)
    r = b.run().results()
    cur = np.array([e[1] / t for e, t in zip(r["electrode_occupation"], r["time"])])
    thr = lambda x: np.exp(x) if x <= 0 else 1.0   # noqa: E731  (exp_tresh, set.py:13-22)
    sg_f = nu * tc[1, 0] * thr((V_S - U_G) / kT)
    gd_f = nu * tc[0, 2] * thr((U_G - 0.0) / kT)
    sg_b = nu * tc[0, 1] * thr((U_G - V_S) / kT)
    gd_b = nu * tc[2, 0] * thr((0.0 - U_G) / kT)
    exact = (sg_f * gd_f - sg_b * gd_b) / (sg_f + gd_f + sg_b + gd_b)
    m, se = cur.mean(), cur.std(ddof=1) / np.sqrt(chains)
    assert abs(m - exact) < 3.5 * se + 1e-12, (m, exact, se)
