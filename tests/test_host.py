"""Host-side logic that needs no GPU."""
import numpy as np
import pytest

from kmc_dn_gb300.engine import make_work_lists, default_lanes
from kmc_dn_gb300.rng import replay_uniforms


def test_work_lists_cover_every_chain_once():
    rng = np.random.default_rng(0)
    S = rng.integers(14, 212, 1000)
    hops = rng.integers(1, 10**6, 1000)
    seen = []
    for G, work, order, smax in make_work_lists(S, hops):
        assert len(work) % max(1, 32 // G) == 0
        ids = work[work >= 0]
        assert np.all([default_lanes(int(S[i])) == G for i in ids])
        assert smax == S[ids].max()
        # within a bin: several chains per warp item sorted by size then hops,
        # one chain per item by work hops x S^2 (all descending)
        if G >= 32:
            key = list(zip(-hops[ids] * S[ids].astype(float) ** 2, -S[ids], -hops[ids]))
        else:
            key = list(zip(-S[ids], -hops[ids]))
        assert key == sorted(key)
        seen.extend(ids.tolist())
    assert sorted(seen) == list(range(1000))


def test_small_launches_get_wider_groups():
    """A launch too small to fill the GPU widens each chain's group (lower
    per-hop latency); a full one keeps the size default."""
    from kmc_dn_gb300.engine import widen_small_launch as w
    assert w(16, 38, 1, 152) == 128            # one N=30 chain: up to 2 x next_pow2(38)
    assert w(32, 128, 1, 152) == 256           # one N=120 chain
    assert w(256, 1008, 1, 152) == 512         # capped at 512 lanes
    assert w(16, 38, 4096, 152) == 16          # the 4096-chain ensemble fills the GPU
    assert w(16, 38, 200, 152) == 64           # 200 x 64 x 2 exceeds a quarter of 152 x 512
    S = np.array([38] * 3 + [128] * 2)
    for G, work, order, smax in make_work_lists(S, np.full(5, 1000), sms=152):
        assert G == (128 if smax == 38 else 256)


def test_short_request_quanta():
    """Long requests run in long-request quanta; a short request runs in one
    launch unless it holds a quarter of the resident threads, when it runs in
    short_big_quantum hops so that its blocks free up for the next one."""
    from kmc_dn_gb300.serving import Request
    s, _ = _admission_server(mem_budget=10**12, long_thread_budget=10**9)
    s.quantum, s.quantum_long, s.short_big_quantum = 20480, 1024, 2048
    assert s._quantum(Request(0, np.zeros((32, 8)), 10**4, 1)) == 20480     # 32 x 64 threads
    assert s._quantum(Request(1, np.zeros((512, 8)), 10**4, 2)) == 2048     # 512 x 64 threads
    assert s._quantum(Request(1, np.zeros((512, 8)), 10**6, 3)) == 1024     # long


def test_balanced_warps_per_block():
    """The launch shape that puts the fewest warps on the busiest SM, with
    every block resident at once (16 warps per SM)."""
    from kmc_dn_gb300.engine import balanced_warps_per_block as bw
    assert bw(2048, 152) == 7          # 293 blocks: at most 14 warps on an SM (8 warps: 16)
    assert bw(1024, 152) == 7          # 147 blocks, one per SM
    assert bw(256, 152) == 4           # spread over more SMs
    assert bw(5000, 152) == 8          # no size fits one wave


def test_work_lists_reject_bad_lanes():
    with pytest.raises(ValueError):
        make_work_lists([38], [10], lanes=6)


def test_replay_stream_open_interval_and_reproducible():
    u = replay_uniforms(123, 100000)
    assert np.all(u > 0) and np.all(u < 1)
    np.testing.assert_array_equal(u, replay_uniforms(123, 100000))
    assert abs(u.mean() - 0.5) < 0.01


def test_native_library_missing_fails_loudly(tmp_path, monkeypatch):
    from kmc_dn_gb300 import _native
    monkeypatch.setattr(_native, "LIB_PATH", str(tmp_path / "nope.so"))
    monkeypatch.setattr(_native, "_LIB", None)
    with pytest.raises(_native.NativeLibraryError):
        _native.lib()


def test_serving_queue_removes_requests_by_identity():
    """Requests carry voltage arrays; removing one from the wait queue must
    not compare arrays (that raised inside the server thread)."""
    from collections import deque
    from kmc_dn_gb300.serving import Request
    a = Request(0, np.zeros((3, 8)), 10, 1, arrival=0.0)
    b = Request(0, np.zeros((5, 8)), 10, 2, arrival=0.0)
    q = deque([a, b])
    q.remove(b)
    assert list(q) == [a] and a != Request(0, np.zeros((3, 8)), 10, 1, arrival=0.0)


def _replica_rank(rank, world, port, out_dir):
    import json
    import os
    import torch.distributed as dist
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.parallel import reduce_step, replica_chains
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        n = 8
        off, sid = replica_chains(rank, n)
        net, V = workloads.homogeneous_ensemble(n + off, 0)
        ms, hops = reduce_step(10.0 * (rank + 1), 1000 * (rank + 1))
        ids = [None] * world
        dist.all_gather_object(ids, sid.tolist())
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump(dict(off=off, sid=sid.tolist(), V=V[off:off + n].tolist(), ms=ms, hops=hops, ids=ids), f)
    finally:
        dist.destroy_process_group()


def test_replicas_over_two_gloo_ranks(tmp_path):
    """The multi-GPU layout (one replica of the ensemble per rank, weak
    scaling) over two gloo ranks on the CPU: disjoint random streams, each
    rank's chains are its slice of one larger ensemble, and the whole-job
    reduction takes the slowest rank's time and every rank's hops."""
    import json
    import socket
    import torch.multiprocessing as mp
    from kmc_dn_gb300 import workloads
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_replica_rank, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    r = [json.load(open(tmp_path / f"rank{k}.json")) for k in range(2)]
    assert set(r[0]["sid"]).isdisjoint(r[1]["sid"])
    assert r[0]["ids"] == r[1]["ids"] == [r[0]["sid"], r[1]["sid"]]
    _, V = workloads.homogeneous_ensemble(16, 0)
    np.testing.assert_array_equal(np.array(r[0]["V"] + r[1]["V"]), V)
    for k in range(2):
        assert r[k]["ms"] == 20.0 and r[k]["hops"] == 3000


def test_autotune_size_classes_and_candidates():
    from kmc_dn_gb300 import autotune
    assert autotune.size_class(20) == 24 and autotune.size_class(38) == 48 and autotune.size_class(212) == 256
    assert autotune.size_class(5000) == 2048
    assert autotune._candidates(38) == [4, 8, 16, 32]
    assert autotune._candidates(212) == [4, 8, 16, 32, 64, 128, 256, 512]
    assert autotune._candidates(1008) == [64, 128, 256, 512]


def test_instrumented_builds_are_exclusive():
    from kmc_dn_gb300 import build
    with pytest.raises(ValueError, match="one of"):
        build.build(debug_checks=True, section_clocks=True)
    assert build.DEBUG_LIB != build.CLOCKS_LIB != build.LIB


def test_hbm_roofline_of_a_launch(tmp_path, monkeypatch):
    """The headline line's HBM roofline: DRAM bytes per launch time against
    the measured copy bandwidth, or the stated fallback without it."""
    import bench
    r = bench.hbm_roofline(2_000_000, 4.0)           # 2 MB in 4 ms = 0.5 GB/s
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and abs(r["achieved"] - 0.5) < 1e-12
    assert r["frac"] == r["achieved"] / r["peak"]
    assert bench.hbm_roofline(None, 4.0) is None
    monkeypatch.setattr(bench, "HERE", str(tmp_path))   # no MEASURED_PEAKS.json there
    r = bench.hbm_roofline(2_000_000, 4.0)
    assert r["peak"] == 6800.0 and "fallback" in r["peak_source"]
    (tmp_path / "MEASURED_PEAKS.json").write_text('{"hbm_gbs": 5000.0}')
    r = bench.hbm_roofline(2_000_000, 4.0)
    assert r["peak"] == 5000.0 and r["peak_source"].startswith("of measured")


def _admission_server(mem_budget, long_thread_budget):
    """A Server with only its admission state (no device): _prepare records
    the admitted request and books its memory, chains and threads."""
    from collections import deque
    from types import SimpleNamespace
    from kmc_dn_gb300.serving import Server, _request_bytes
    s = object.__new__(Server)
    s.networks = [SimpleNamespace(N=30, P=8), SimpleNamespace(N=240, P=8)]
    s.queue, s.active, s.admitted = deque(), [], []
    s.lanes, s.short_lanes_factor, s.short_hops = None, 4, 20000
    s.short_thread_cap = 152 * 512 // 2
    s.mem_budget, s.mem_used = mem_budget, 0
    s.max_active_chains, s.active_chains = 16384, 0
    s.long_thread_budget, s.active_long_threads = long_thread_budget, 0

    def prepare(req, need):
        s.admitted.append(req)
        s.active.append(req)
        s.mem_used += need
        s.active_chains += req.voltages.shape[0]
        if req.hops > s.short_hops:
            s.active_long_threads += s._threads(req)
    s._prepare = prepare
    return s, _request_bytes


def test_admission_least_work_first_within_the_memory_budget():
    from kmc_dn_gb300.serving import Request
    s, nbytes = _admission_server(mem_budget=10**12, long_thread_budget=10**9)
    big = Request(1, np.zeros((512, 8)), 10**6, 1)
    small = Request(0, np.zeros((32, 8)), 10**4, 2)
    mid = Request(0, np.zeros((512, 8)), 10**5, 3)
    s.queue.extend([big, small, mid])
    s._admit()
    assert s.admitted == [small, mid, big]          # least chains x hops x pairs first
    # a budget that holds the first two only: the third waits
    s, nbytes = _admission_server(mem_budget=nbytes(32, 30, 8) + nbytes(512, 30, 8), long_thread_budget=10**9)
    s.queue.extend([big, small, mid])
    s._admit()
    assert s.admitted == [small, mid] and list(s.queue) == [big]


def test_admission_caps_long_requests_but_not_short_ones():
    """Long requests may hold only the long-thread budget; a short request
    behind them is still admitted on arrival."""
    from kmc_dn_gb300.engine import default_lanes
    from kmc_dn_gb300.serving import Request
    threads = 512 * default_lanes(248)               # one 512-chain N=240 long request
    s, _ = _admission_server(mem_budget=10**12, long_thread_budget=int(1.5 * threads))
    long_a = Request(1, np.zeros((512, 8)), 10**6, 1)
    long_b = Request(1, np.zeros((512, 8)), 10**6, 2)
    short = Request(1, np.zeros((512, 8)), 10**4, 3)
    s.queue.extend([long_a, long_b])
    s._admit()
    assert s.admitted == [long_a] and list(s.queue) == [long_b]   # the second would exceed the budget
    s.queue.append(short)
    s._admit()
    assert s.admitted == [long_a, short] and list(s.queue) == [long_b]


def test_short_request_groups_narrow_to_leave_room():
    """A short request widens its groups (lower latency) only while its
    chains hold at most the short-thread cap; a large one narrows below the
    default, so that the next short request finds free SMs."""
    from kmc_dn_gb300.engine import default_lanes
    from kmc_dn_gb300.serving import Request
    s, _ = _admission_server(mem_budget=10**12, long_thread_budget=10**9)
    cap = s.short_thread_cap
    small = Request(0, np.zeros((32, 8)), 10**4, 1)          # N=30: 16 x 4 lanes
    assert s._lanes(small) == 4 * default_lanes(38)
    big = Request(1, np.zeros((512, 8)), 10**4, 2)           # N=240: 512 chains
    G = s._lanes(big)
    assert 512 * G <= cap and 512 * 2 * G > cap
    assert s._lanes(Request(1, np.zeros((512, 8)), 10**6, 3)) is None   # long: the default


def test_prune_cut_is_taken_in_float32_as_go_does():
    """simulation.go:199-215 keeps tc > cut * max(tc) with tc, the cut and
    their product in float32: an entry a hair above the cut in FP64 that
    rounds onto it in float32 is pruned, as in Go."""
    from kmc_dn_gb300.engine import prune
    tc = np.array([[0.0, 1.0, 0.1 + 1e-12], [1.0, 0.0, 0.25], [0.1 + 1e-12, 0.25, 0.0]])
    p = prune(tc, 0.1)
    assert p[0, 2] == 0.0 and p[2, 0] == 0.0          # float32(0.1 + 1e-12) == float32(0.1): not above
    assert p[0, 1] == 1.0 and p[1, 2] == 0.25         # clearly above: kept with its FP64 value
    np.testing.assert_array_equal(prune(tc, 0.0), tc)  # no cut: unchanged


def test_long_requests_pause_while_short_ones_run():
    """Strict priority: a long request gets no new quantum while a short one
    is waiting or active, until the starvation guard lets one through."""
    from kmc_dn_gb300.serving import Request
    s, _ = _admission_server(mem_budget=10**12, long_thread_budget=10**9)
    s.max_long_pause = 0.5
    long_ = Request(1, np.zeros((64, 8)), 10**6, 1)
    short = Request(0, np.zeros((32, 8)), 10**4, 2)
    assert not s._short_busy()
    assert s._may_launch(long_, s._short_busy(), now=0.0)
    s.queue.append(short)
    busy = s._short_busy()
    assert busy
    assert s._may_launch(short, busy, now=1.0)             # short ones always launch
    assert not s._may_launch(long_, busy, now=1.0)          # paused from t = 1.0
    assert not s._may_launch(long_, busy, now=1.4)
    assert s._may_launch(long_, busy, now=1.6)              # held back > 0.5 s: one quantum
    assert not s._may_launch(long_, busy, now=1.7)          # and paused again
    s.queue.clear()
    short.launched_hops = short.hops
    s.active = [short]                                      # short work all launched: not busy
    assert not s._short_busy() and s._may_launch(long_, False, now=2.0)
