"""kmc_engine_*: chain state resident on the device between runs.  A run
split over several kmc_engine_run calls must give exactly the results of one
kmc_run_batch_host call with the same inputs and seed; record mode reads the
cumulative sums."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(n=24, hops=5000, seed=3):
    from kmc_dn_gb300 import workloads
    rng = np.random.default_rng(seed)
    nets = [workloads.plain_network(0), workloads.plain_network(1)]
    geoms = []
    d, tc, off = [], [], 0
    for net in nets:
        geoms.append((net.N, net.P, net.nu, net.I_0, net.R, off))
        d.append(net.distances.ravel())
        tc.append(net.transitions_constant.ravel())
        off += net.S * net.S
    cg = rng.integers(0, 2, n).astype(np.int32)
    V = rng.uniform(-1, 1, (n, 8))
    ec = np.concatenate([nets[g].E_constant(V[c]) for c, g in enumerate(cg)])
    se = np.concatenate([nets[g].site_energies(V[c]) for c, g in enumerate(cg)])
    occ = np.concatenate([nets[g].occupation.astype(np.uint8) for g in cg])
    return dict(nets=nets, geoms=geoms, d=np.concatenate(d), tc=np.concatenate(tc), cg=cg, ec=ec, se=se,
                occ=occ, hops=np.full(n, hops, np.int64), kT=np.ones(n), n=n)


def _arrays(x):
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    g = x["geoms"]
    gN = np.array([t[0] for t in g], np.int32)
    gP = np.array([t[1] for t in g], np.int32)
    gnu = np.array([t[2] for t in g])
    gI = np.array([t[3] for t in g])
    gR = np.array([t[4] for t in g])
    goff = np.array([t[5] for t in g], np.int64)
    keep = [gN, gP, gnu, gI, gR, goff]
    return p, keep, [len(g), p(gN), p(gP), p(gnu), p(gI), p(gR), p(goff), p(x["d"]), p(x["tc"]), x["n"],
                     p(x["cg"]), p(x["kT"]), p(x["ec"]), p(x["se"])]


def test_engine_split_run_equals_one_host_call(engine_lib):
    from kmc_dn_gb300._native import check, lib
    L = lib()
    x = _inputs()
    n = x["n"]
    P = sum(x["nets"][g].P for g in x["cg"])
    N = sum(x["nets"][g].N for g in x["cg"])
    # one host call
    p, keep, head = _arrays(x)
    occ1 = x["occ"].copy()
    t1, eo1, st1 = np.zeros(n), np.zeros(P, np.int64), np.zeros(n, np.int32)
    check(L.kmc_run_batch_host(*head, p(occ1), p(x["hops"]), 77, 16, p(t1), p(eo1), p(st1)))
    # the same through the engine handle, in three runs
    h = C.c_void_p()
    check(L.kmc_engine_create(C.byref(h), *head, p(x["occ"]), p(x["hops"]), 77, 16, 0, None))
    try:
        for seg in (1024, 2048, 0):
            check(L.kmc_engine_run(h, seg))
        t2, eo2, st2 = np.zeros(n), np.zeros(P, np.int64), np.zeros(n, np.int32)
        occ2, hd = np.zeros(N, np.uint8), np.zeros(n, np.int64)
        check(L.kmc_engine_read(h, p(t2), p(eo2), p(occ2), p(st2), p(hd), None, None))
    finally:
        L.kmc_engine_destroy(h)
    assert (st1 == 0).all() and (st2 == 0).all() and (hd == 5000).all()
    np.testing.assert_array_equal(t1, t2)
    np.testing.assert_array_equal(eo1, eo2)
    np.testing.assert_array_equal(occ1, occ2)


def test_engine_record_mode_reads_cumulative_sums(engine_lib):
    from kmc_dn_gb300._native import RECORD_GO, check, lib
    L = lib()
    x = _inputs(n=4, hops=3000)
    n = x["n"]
    S = [x["nets"][g].S for g in x["cg"]]
    N = [x["nets"][g].N for g in x["cg"]]
    P = [x["nets"][g].P for g in x["cg"]]
    p, keep, head = _arrays(x)
    h = C.c_void_p()
    check(L.kmc_engine_create(C.byref(h), *head, p(x["occ"]), p(x["hops"]), 5, 16, RECORD_GO, None))
    try:
        check(L.kmc_engine_run(h, 0))
        t = np.zeros(n)
        eo = np.zeros(sum(P), np.int64)
        tr = np.zeros(sum(s * s for s in S))
        oit = np.zeros(sum(N))
        check(L.kmc_engine_read(h, p(t), p(eo), None, None, None, p(tr), p(oit)))
    finally:
        L.kmc_engine_destroy(h)
    to, eoff, so = 0, 0, 0
    for c in range(n):
        T = tr[to:to + S[c] ** 2].reshape(S[c], S[c])
        np.testing.assert_array_equal(T, -T.T)                       # Go convention: net traffic
        np.testing.assert_array_equal(eo[eoff:eoff + P[c]], T[:, N[c]:].sum(axis=0))
        assert np.all(oit[so:so + N[c]] >= 0) and np.all(oit[so:so + N[c]] <= t[c] * (1 + 1e-12))
        to += S[c] ** 2
        eoff += P[c]
        so += N[c]
