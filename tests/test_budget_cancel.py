"""Failure detection without a GPU fault: the engine's wall-clock budget
(KMC_ERR_TIMEOUT) and host-mapped cancel word (KMC_ERR_CANCELLED) stop chains
at a 1024-hop boundary with their state consistent, a later launch resumes
them as if uninterrupted, and the serving loop cancels requests and refuses
non-finite inputs.  Every launch here also carries a time budget,
so no kernel can run long even if a stop signal were missed."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(n, hops, seed=4):
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    net = workloads.plain_network(0)
    rng = np.random.default_rng(seed)
    V = rng.uniform(-1, 1, (n, net.P))
    spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
    return Batch([spec], np.zeros(n, np.int32), np.full(n, net.kT), [net.E_constant(v) for v in V], list(V),
                 np.tile(net.occupation.astype(np.uint8), (n, 1)), np.full(n, hops), seed=seed, lanes=16)


def _same(a, b):
    for k in ("time", "hops_done", "status"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    for k in ("electrode_occupation", "occupation"):
        for x, y in zip(a[k], b[k]):
            np.testing.assert_array_equal(x, y, err_msg=k)


def test_time_budget_stops_and_a_later_launch_resumes_identically(engine_lib):
    from kmc_dn_gb300._native import KMC_ERR_TIMEOUT
    hops = 200_000
    a = _batch(64, hops)
    a.time_budget_ns = 3_000_000                 # 3 ms: far less than the run needs
    a.run()
    r = a.results()
    assert (r["status"] == KMC_ERR_TIMEOUT).all()
    assert (r["hops_done"] % 1024 == 0).all() and (r["hops_done"] >= 1024).all() and (r["hops_done"] < hops).all()
    a.time_budget_ns = 0
    a.run()
    r = a.results()
    assert (r["status"] == 0).all() and (r["hops_done"] == hops).all()
    b = _batch(64, hops)
    b.run()
    _same(r, b.results())


def test_cancel_word_stops_a_running_launch(engine_lib):
    import torch
    from kmc_dn_gb300._native import KMC_ERR_CANCELLED
    from kmc_dn_gb300.engine import CancelWord
    w = CancelWord()
    try:
        b = _batch(64, 10**8)
        b.cancel = w
        b.time_budget_ns = 3_000_000_000         # safety net: 3 s
        st = torch.cuda.Stream()
        t0 = time.perf_counter()
        b.launch(stream=st)
        time.sleep(0.05)
        w.set()
        st.synchronize()
        dt = time.perf_counter() - t0
        r = b.results()
        assert (r["status"] == KMC_ERR_CANCELLED).all()
        assert (r["hops_done"] % 1024 == 0).all() and (r["hops_done"] > 0).all()
        assert dt < 1.5, dt                       # stopped by the word, not by the safety net
        # cleared: the chains continue from where they stopped
        w.clear()
        before = r["hops_done"].copy()
        b.launch(4096)
        r = b.results()
        assert (r["status"] == 0).all() and (r["hops_done"] == before + 4096).all()
    finally:
        w.close()


def test_cancel_before_launch_runs_nothing(engine_lib):
    from kmc_dn_gb300._native import KMC_ERR_CANCELLED
    from kmc_dn_gb300.engine import CancelWord
    w = CancelWord()
    try:
        w.set()
        b = _batch(8, 5000)
        b.cancel = w
        b.time_budget_ns = 3_000_000_000
        r = b.run().results()
        assert (r["status"] == KMC_ERR_CANCELLED).all() and (r["hops_done"] == 0).all()
    finally:
        w.close()


def test_serving_cancels_and_refuses_nonfinite_inputs(engine_lib):
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300._native import KMC_ERR_CANCELLED
    from kmc_dn_gb300.serving import Server
    nets = workloads.serving_geometries(seed=0, sizes=(30,))
    srv = Server(nets, quantum=4096, quantum_long=4096)
    srv.start()
    try:
        long_req = srv.submit(0, np.zeros((64, 8)), 10**9, seed=1)       # would run for hours
        waiting = srv.submit(0, np.zeros((8, 8)), 10**9, seed=2)
        V = np.random.default_rng(0).uniform(-1, 1, (4, 8))
        V[2, 3] = np.nan
        # a NaN energy difference reads as downhill in the hop loop (as in the
        # reference, kmc_dopant_networks.py:74-82): the server refuses it
        with pytest.raises(ValueError, match="finite"):
            srv.submit(0, V, 3000, seed=3)
        ok = srv.submit(0, np.nan_to_num(V), 3000, seed=3)
        time.sleep(0.2)
        assert srv.cancel(long_req) and srv.cancel(waiting)
        r = long_req.future.result(timeout=10)
        assert r["cancelled"] and (r["status"] == KMC_ERR_CANCELLED).all()
        assert waiting.future.result(timeout=10)["cancelled"]
        ro = ok.future.result(timeout=30)
        assert not ro["cancelled"] and (ro["status"] == 0).all() and (ro["hops_done"] == 3000).all()
    finally:
        srv.stop(drain=True)
