"""The continuous-batching server: results independent of the mix, requests
admitted while others run, latency records."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _server(**kw):
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.serving import Server
    nets = workloads.serving_geometries(seed=0, sizes=(30, 60))
    return Server(nets, **kw), nets


def test_result_same_alone_and_in_the_mix(engine_lib):
    srv, nets = _server(quantum=2048)
    rng = np.random.default_rng(0)
    V = rng.uniform(-1, 1, (32, 8))
    a = srv.submit(0, V, 5000, seed=42)
    srv.run_sync()
    alone = a.future.result()
    # the same request among others of both geometries and budgets, arriving
    # while earlier ones are still running
    srv.start()
    others = [srv.submit(g, rng.uniform(-1, 1, (64, 8)), h, seed=s)
              for g, h, s in ((1, 20000, 1), (0, 3000, 2), (1, 7000, 3))]
    time.sleep(0.01)
    b = srv.submit(0, V, 5000, seed=42)
    more = [srv.submit(0, rng.uniform(-1, 1, (16, 8)), 9000, seed=5)]
    srv.stop(drain=True)
    mix = b.future.result()
    np.testing.assert_array_equal(alone["time"], mix["time"])
    np.testing.assert_array_equal(alone["electrode_occupation"], mix["electrode_occupation"])
    assert np.all(mix["status"] == 0)
    for r in others + more:
        assert np.all(r.future.result()["status"] == 0)
    assert mix["latency"] > 0


def test_admission_respects_memory_budget(engine_lib):
    from kmc_dn_gb300.serving import _request_bytes
    srv, nets = _server(quantum=1024, mem_budget=_request_bytes(64, 60, 8) + 1)
    reqs = [srv.submit(1, np.zeros((64, 8)), 2048, seed=i) for i in range(3)]
    peak = 0
    torch_ok = True
    while True:
        with srv.lock:
            srv._admit()
            peak = max(peak, len(srv.active))
            if not srv.queue and not srv.active:
                break
        srv._launch_ready()
        srv._collect()
    assert peak == 1 and torch_ok
    assert all(np.all(r.future.result()["status"] == 0) for r in reqs)


def test_latency_summary(engine_lib):
    from kmc_dn_gb300.serving import latency_summary
    srv, nets = _server(quantum=2048)
    reqs = [srv.submit(0, np.zeros((8, 8)), 2000 if i % 2 else 4000, seed=i) for i in range(6)]
    srv.run_sync()
    s = latency_summary(reqs)
    assert s["all"]["n"] == 6 and s["hops_2000"]["n"] == 3
    assert s["all"]["p99_ms"] >= s["all"]["p50_ms"] > 0


def test_short_requests_bypass_the_long_request_budget(engine_lib):
    """Long requests hold at most their share of the device's thread slots; a
    short request is admitted beside them at once."""
    srv, nets = _server(quantum=2048, short_hops=4096)
    srv.long_thread_budget = 64 * 16        # room for one 64-chain request of 16 lanes
    longs = [srv.submit(0, np.zeros((64, 8)), 8192, seed=i) for i in range(2)]
    short = srv.submit(0, np.zeros((16, 8)), 2048, seed=9)
    with srv.lock:
        srv._admit()
        admitted = set(id(r) for r in srv.active)
    assert id(short) in admitted and id(longs[0]) in admitted and id(longs[1]) not in admitted
    assert srv.active_long_chains == 64
    srv.run_sync()
    assert all(np.all(r.future.result()["status"] == 0) for r in longs + [short])
    assert srv.active_long_chains == 0 and srv.active_chains == 0
