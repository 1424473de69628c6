"""GPU parity: the CUDA kernels against the oracle and the reference's golden
replays.  Every test here runs on the device through the C ABI."""
import numpy as np
import pytest

from conftest import golden_files, load_golden
from kmc_dn_gb300.rng import replay_uniforms

pytestmark = pytest.mark.gpu

REPLAYS = golden_files("replay_*.npz")


def _f64(g, hops=None, uniforms=None, seed=0, record=True, hop_log=True, occupation=None):
    from kmc_dn_gb300.engine import simulate_f64
    hops = int(g["hops"]) if hops is None else hops
    return simulate_f64(int(g["N"]), int(g["P"]), float(g["nu"]), float(g["kT"]), float(g["I_0"]),
                        float(g["R"]), g["occupation"] if occupation is None else occupation,
                        g["distances"], g["E_constant"], g["site_energies"], g["transitions_constant"],
                        hops, record=record, uniforms=uniforms, seed=seed, hop_log=hop_log)


@pytest.mark.parametrize("path", REPLAYS, ids=lambda p: p.split("replay_")[-1][:-4])
def test_f64_kernel_replays_reference(engine_lib, path):
    """Bit-exact hop sequence of the reference's own loop on the same stream
    (1e5 hops for the two long cases)."""
    g = load_golden(path)
    hops = int(g["hops"])
    u = replay_uniforms(int(g["seed"]), 2 * hops)
    r = _f64(g, uniforms=u)
    assert r["status"] == 0
    log = r["hop_log"]
    ref = g["hop_log"].astype(np.int32)
    mism = np.flatnonzero(np.any(log != ref, axis=1))
    assert mism.size == 0, f"first divergence at hop {mism[0]} of {hops}"
    np.testing.assert_array_equal(r["electrode_occupation"], g["final_electrode_occupation"])
    np.testing.assert_array_equal(r["occupation"].astype(np.uint8), g["final_occupation"])
    np.testing.assert_array_equal(r["traffic"], g["traffic"])
    assert abs(r["time"] - float(g["time"])) <= 1e-11 * abs(float(g["time"]))
    np.testing.assert_allclose(r["occupations_in_time"], g["occupations_in_time"], rtol=1e-11)


def test_f64_kernel_matches_oracle_fresh_seeds(engine_lib, oracle_mod):
    from kmc_dn_gb300 import workloads
    net = workloads.plain_network(3)
    for seed in (21, 22):
        hops = 5000
        u = replay_uniforms(seed, 2 * hops)
        g = dict(N=net.N, P=net.P, nu=net.nu, kT=net.kT, I_0=net.I_0, R=net.R,
                 occupation=net.occupation.astype(np.uint8), distances=net.distances,
                 E_constant=net.E_constant(), site_energies=net.site_energies(),
                 transitions_constant=net.transitions_constant)
        r = _f64(g, hops=hops, uniforms=u)
        o = oracle_mod.numba_replay(net.N, net.P, net.nu, net.kT, net.I_0, net.R, g["occupation"],
                                    net.distances, g["E_constant"], g["site_energies"],
                                    net.transitions_constant, u, record=True)
        np.testing.assert_array_equal(r["hop_log"], o["hop_log"])
        assert abs(r["time"] - o["time"]) <= 1e-11 * o["time"]


def test_f64_philox_mode_runs(engine_lib):
    g = load_golden([p for p in REPLAYS if "plain" in p][0])
    a = _f64(g, hops=2000, seed=5, record=False, hop_log=True)
    b = _f64(g, hops=2000, seed=5, record=False, hop_log=True)
    c = _f64(g, hops=2000, seed=6, record=False, hop_log=True)
    assert a["status"] == 0
    np.testing.assert_array_equal(a["hop_log"], b["hop_log"])     # deterministic per seed
    assert np.any(a["hop_log"] != c["hop_log"])


def _batch_one(g, hops, uniforms=None, record=0, lanes=8, seed=0, pair_mode="table", spec=None):
    from kmc_dn_gb300.engine import Batch, TableSpec
    N, P = int(g["N"]), int(g["P"])
    if spec is None:
        spec = TableSpec(N, P, float(g["nu"]), float(g["I_0"]), float(g["R"]), g["distances"],
                         g["transitions_constant"])
    se = np.asarray(g["site_energies"], np.float64)
    b = Batch([spec], [0], [float(g["kT"])], [g["E_constant"]], [se[N:]], [g["occupation"]], [hops],
              seed=seed, record=record, lanes=lanes,
              replay=[uniforms] if uniforms is not None else None, pair_mode=pair_mode)
    b.run()
    return b.results()


@pytest.mark.parametrize("lanes,pair_mode", [(4, "table"), (8, "table"), (16, "table"), (32, "table"),
                                              (64, "table"), (128, "table"), (16, "positions"),
                                              (32, "positions"), (128, "positions")])
def test_f32_engine_replay_agrees_where_margins_allow(engine_lib, oracle_mod, lanes, pair_mode):
    """Fed the same stream, the FP32 engine picks the reference's pair on every
    hop whose event uniform is further than 1e-4 (relative) from a cumulative
    boundary; the sequences may part only after the first closer call."""
    g = load_golden([p for p in REPLAYS if "plain" in p][0])
    hops = 4000
    u = replay_uniforms(int(g["seed"]), 2 * hops)
    o = oracle_mod.numba_replay(int(g["N"]), int(g["P"]), float(g["nu"]), float(g["kT"]),
                                float(g["I_0"]), float(g["R"]), g["occupation"], g["distances"],
                                g["E_constant"], g["site_energies"], g["transitions_constant"], u,
                                hops=hops, record=True)
    close = np.flatnonzero(o["margins"] < 1e-4)
    safe = int(close[0]) if close.size else hops
    assert safe > 50
    spec = None
    if pair_mode == "positions":
        from kmc_dn_gb300 import workloads
        from kmc_dn_gb300.engine import TableSpec
        spec = TableSpec.from_network(workloads.plain_network(0))   # the golden's network
        np.testing.assert_array_equal(spec.distances, g["distances"])
    r = _batch_one(g, safe, uniforms=u, record=1, lanes=lanes, pair_mode=pair_mode, spec=spec)
    assert r["status"][0] == 0
    # the final state after `safe` hops equals the oracle's state after `safe` hops
    o2 = oracle_mod.numba_replay(int(g["N"]), int(g["P"]), float(g["nu"]), float(g["kT"]),
                                 float(g["I_0"]), float(g["R"]), g["occupation"], g["distances"],
                                 g["E_constant"], g["site_energies"], g["transitions_constant"], u,
                                 hops=safe, record=True)
    np.testing.assert_array_equal(r["occupation"][0], o2["occupation"].astype(bool))
    np.testing.assert_array_equal(r["electrode_occupation"][0], o2["electrode_occupation"])
    np.testing.assert_array_equal(r["traffic"][0], o2["traffic"].astype(np.int32))
    assert abs(r["time"][0] - o2["time"]) <= 1e-4 * o2["time"]
    np.testing.assert_allclose(r["occ_time"][0], o2["occupations_in_time"], rtol=1e-4,
                               atol=1e-4 * o2["time"])


def test_f32_engine_same_alone_and_in_the_mix(engine_lib):
    """A chain's result does not depend on which other chains share its launch."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    nets = [workloads.plain_network(s) for s in (1, 2)]
    specs = [TableSpec(n.N, n.P, n.nu, n.I_0, n.R, n.distances, n.transitions_constant) for n in nets]
    hops = 6000

    def run(chains):
        b = Batch(specs, [c[0] for c in chains], [1.0] * len(chains),
                  [nets[c[0]].E_constant() for c in chains],
                  [nets[c[0]].electrodes[:, 3] for c in chains],
                  [nets[c[0]].occupation.astype(np.uint8) for c in chains],
                  [c[1] for c in chains], streams=[c[2] for c in chains], seed=77, lanes=8)
        b.run()
        return b.results()
    alone = run([(0, hops, 5)])
    mix = run([(1, 3000, 9), (0, 1000, 4), (0, hops, 5), (1, hops, 11), (0, 2500, 3)])
    assert alone["status"][0] == 0
    assert mix["time"][2] == alone["time"][0]
    np.testing.assert_array_equal(mix["electrode_occupation"][2], alone["electrode_occupation"][0])
    np.testing.assert_array_equal(mix["occupation"][2], alone["occupation"][0])


@pytest.mark.parametrize("lanes", [8, 16, 32])
def test_f32_engine_register_variants_identical(engine_lib, lanes):
    """A small launch runs the register-rich warp-slice variant (every block
    resident at 2 per SM), a launch of many chains the 85-register one; the
    same chain gives the same bits in both."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    n = workloads.plain_network(0)
    spec = TableSpec(n.N, n.P, n.nu, n.I_0, n.R, n.distances, n.transitions_constant)
    rng = np.random.default_rng(8)

    def run(n_chains, V):
        b = Batch([spec], np.zeros(n_chains, np.int32), np.full(n_chains, n.kT), [n.E_constant(v) for v in V],
                  list(V), np.tile(n.occupation.astype(np.uint8), (n_chains, 1)), np.full(n_chains, 3000),
                  seed=21, lanes=lanes, warps_per_block=8, record=2)
        return b.run().results()
    big = 16 * 152 * 32 // lanes + 64          # more warps than the SMs hold at 16 each
    V = rng.uniform(-1, 1, (big, n.P))
    small = run(48, V[:48])
    large = run(big, V)
    assert (small["status"] == 0).all() and (large["status"] == 0).all()
    np.testing.assert_array_equal(small["time"], large["time"][:48])
    for k in ("electrode_occupation", "occupation", "traffic", "occ_time"):
        for x, y in zip(small[k], large[k][:48]):
            np.testing.assert_array_equal(x, y)


def test_f32_engine_split_launches_identical(engine_lib):
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    n = workloads.plain_network(4)
    spec = TableSpec(n.N, n.P, n.nu, n.I_0, n.R, n.distances, n.transitions_constant)

    def mk():
        return Batch([spec], [0, 0], [1.0, 1.0], [n.E_constant()] * 2, [n.electrodes[:, 3]] * 2,
                     [n.occupation.astype(np.uint8)] * 2, [8192, 8192], seed=3, lanes=8, record=2)
    a = mk().launch(8192).results()
    b = mk()
    for _ in range(4):
        b.launch(2048)
    b = b.results()
    np.testing.assert_array_equal(a["time"], b["time"])
    for k in ("electrode_occupation", "occupation", "traffic", "occ_time"):
        for x, y in zip(a[k], b[k]):
            np.testing.assert_array_equal(x, y)
    assert list(b["hops_done"]) == [8192, 8192]


def test_f32_engine_statistics_vs_fp64_oracle(engine_lib, oracle_mod):
    """Electrode currents of the FP32 engine agree with the FP64 oracle within
    3 sigma of their Monte Carlo error (independent seeds on both sides)."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    n = workloads.plain_network(0)
    hops = 100_000
    reps_gpu, reps_cpu = 256, 16
    spec = TableSpec(n.N, n.P, n.nu, n.I_0, n.R, n.distances, n.transitions_constant)
    b = Batch([spec], [0] * reps_gpu, [1.0] * reps_gpu, [n.E_constant()] * reps_gpu,
              [n.electrodes[:, 3]] * reps_gpu, [n.occupation.astype(np.uint8)] * reps_gpu,
              [hops] * reps_gpu, seed=1234, lanes=8)
    b.run()
    r = b.results()
    assert np.all(r["status"] == 0)
    cur32 = np.array([e / t for e, t in zip(r["electrode_occupation"], r["time"])])
    cur64 = []
    for s in range(reps_cpu):
        u = replay_uniforms(9000 + s, 2 * hops)
        o = oracle_mod.numba_replay(n.N, n.P, n.nu, n.kT, n.I_0, n.R, n.occupation.astype(np.uint8),
                                    n.distances, n.E_constant(), n.site_energies(),
                                    n.transitions_constant, u, record=False)
        cur64.append(o["electrode_occupation"] / o["time"])
    cur64 = np.array(cur64)
    m32, m64 = cur32.mean(0), cur64.mean(0)
    sig = np.sqrt(cur32.var(0, ddof=1) / reps_gpu + cur64.var(0, ddof=1) / reps_cpu)
    z = np.abs(m32 - m64) / sig
    assert np.all(z < 3.0), (z, m32, m64)


def test_run_batch_host_matches_device_batch(engine_lib):
    """The host-buffer C entry point gives the device-buffer path's results."""
    import ctypes as C
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300._native import lib, check
    from kmc_dn_gb300.engine import Batch, TableSpec
    n = workloads.plain_network(2)
    nc, hops, seed = 24, 3000, 99
    V = np.random.default_rng(0).uniform(-1, 1, (nc, n.P))
    ec = np.concatenate([n.E_constant(v) for v in V])
    se = np.concatenate([np.concatenate([np.zeros(n.N), v]) for v in V])
    occ = np.tile(n.occupation.astype(np.uint8), nc)
    t_out = np.zeros(nc)
    eo = np.zeros(nc * n.P, np.int64)
    st = np.zeros(nc, np.int32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(lib().kmc_run_batch_host(1, p(np.array([n.N], np.int32)), p(np.array([n.P], np.int32)),
                                   p(np.array([n.nu])), p(np.array([n.I_0])), p(np.array([n.R])),
                                   p(np.array([0], np.int64)), p(np.ascontiguousarray(n.distances)),
                                   p(np.ascontiguousarray(n.transitions_constant)), nc,
                                   p(np.zeros(nc, np.int32)), p(np.ones(nc)), p(ec), p(se), p(occ),
                                   p(np.full(nc, hops, np.int64)), seed, 8, p(t_out), p(eo), p(st)))
    spec = TableSpec(n.N, n.P, n.nu, n.I_0, n.R, n.distances, n.transitions_constant)
    b = Batch([spec], [0] * nc, [1.0] * nc, [n.E_constant(v) for v in V], list(V),
              [n.occupation.astype(np.uint8)] * nc, [hops] * nc, seed=seed, lanes=8)
    r = b.run().results()
    np.testing.assert_array_equal(st, 0)
    np.testing.assert_array_equal(t_out, r["time"])
    np.testing.assert_array_equal(eo.reshape(nc, n.P), np.array(r["electrode_occupation"]))


def test_no_allowed_transition_reports_status(engine_lib):
    """A closed single-site system has no allowed hop: the chain stops with
    KMC_ERR_NONFINITE instead of producing NaN times (the reference divides
    by a zero total rate)."""
    from kmc_dn_gb300.engine import Batch, TableSpec, simulate_f64
    from kmc_dn_gb300._native import KMC_ERR_NONFINITE
    d = np.zeros((1, 1))
    tc = np.zeros((1, 1))
    r = simulate_f64(1, 0, 1.0, 1.0, 1.0, 1.0, [1], d, [0.0], [0.0], tc, 10)
    assert r["status"] == KMC_ERR_NONFINITE
    b = Batch([TableSpec(1, 0, 1.0, 1.0, 1.0, d, tc)], [0], [1.0], [[0.0]], [[]], [[1]], [10], lanes=4)
    assert b.run().results()["status"][0] == KMC_ERR_NONFINITE


@pytest.mark.parametrize("lanes,pair_mode", [(32, "table"), (128, "table"), (128, "positions"),
                                              (256, "positions")])
def test_f32_engine_large_network_replay(engine_lib, oracle_mod, lanes, pair_mode):
    """A 300-acceptor network (block groups, multi-word occupancy bitmask):
    the engine follows the FP64 oracle over the hops whose margins allow."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import TableSpec
    net = workloads.large_network(seed=3, N=300, M=30)
    hops = 400
    u = replay_uniforms(50, 2 * hops)
    occ = net.occupation.astype(np.uint8)
    o = oracle_mod.numba_replay(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances,
                                net.E_constant(), net.site_energies(), net.transitions_constant, u,
                                hops=hops, record=False)
    close = np.flatnonzero(o["margins"] < 1e-4)
    safe = int(close[0]) if close.size else hops
    assert safe >= 20
    o2 = oracle_mod.numba_replay(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances,
                                 net.E_constant(), net.site_energies(), net.transitions_constant, u,
                                 hops=safe, record=False)
    g = dict(N=net.N, P=net.P, nu=net.nu, kT=net.kT, I_0=net.I_0, R=net.R, occupation=occ,
             distances=net.distances, E_constant=net.E_constant(), site_energies=net.site_energies(),
             transitions_constant=net.transitions_constant)
    r = _batch_one(g, safe, uniforms=u, lanes=lanes, pair_mode=pair_mode,
                   spec=TableSpec.from_network(net))
    assert r["status"][0] == 0
    np.testing.assert_array_equal(r["occupation"][0], o2["occupation"].astype(bool))
    np.testing.assert_array_equal(r["electrode_occupation"][0], o2["electrode_occupation"])
    assert abs(r["time"][0] - o2["time"]) <= 1e-4 * o2["time"]


def test_positions_mode_rejects_inconsistent_tables(engine_lib):
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    net = workloads.plain_network(0)
    spec = TableSpec.from_network(net)
    spec.transitions_constant = spec.transitions_constant * 1.5     # e.g. ab changed, tc not recomputed
    spec.from_positions = False                                      # caller-supplied tables: verified
    with pytest.raises(ValueError):
        Batch([spec], [0], [1.0], [net.E_constant()], [net.electrodes[:, 3]],
              [net.occupation.astype(np.uint8)], [10], pair_mode="positions")


@pytest.mark.parametrize("pair_mode", ["positions", "table"])
def test_largest_network_runs(engine_lib, pair_mode):
    """S = 2048 sites (the engine's limit: pair indices stay below 2^22) with
    64 electrodes (the electrode limit), block groups of 512."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    N, P = 2048 - 64, 64
    rng = np.random.Generator(np.random.PCG64(5))
    L = float(np.sqrt(N / workloads.DENSITY))
    net = workloads.make_network(rng, N, N // 10, L, L, workloads.perimeter_electrodes(L, P),
                                 voltages=rng.uniform(-1, 1, P), I_0=50.0)
    spec = TableSpec.from_network(net) if pair_mode == "positions" else \
        TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
    b = Batch([spec], [0, 0], [1.0, 1.0], [net.E_constant()] * 2, [net.electrodes[:, 3]] * 2,
              [net.occupation.astype(np.uint8)] * 2, [300, 300], lanes=512, pair_mode=pair_mode, seed=3)
    r = b.run().results()
    assert (r["status"] == 0).all() and (r["hops_done"] == 300).all() and (r["time"] > 0).all()
    # holes are conserved up to what the electrodes absorbed
    for c in range(2):
        assert int(r["occupation"][c].sum()) - int(net.occupation.sum()) == -int(r["electrode_occupation"][c].sum())


def test_sizes_beyond_the_limits_are_rejected(engine_lib):
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300._native import KmcError
    from kmc_dn_gb300.engine import Batch, TableSpec
    # 2049 sites: refused before any launch
    N, P = 2049 - 8, 8
    S = N + P
    d = np.ones((S, S))
    np.fill_diagonal(d, 0.0)
    spec = TableSpec(N, P, 1.0, 1.0, 1.0, d, np.zeros((S, S)))
    with pytest.raises(KmcError):
        Batch([spec], [0], [1.0], [np.zeros(N)], [np.zeros(P)], [np.zeros(N, np.uint8)], [10],
              lanes=512).run()
    # 65 electrodes: refused by the host before any launch (the kernel would
    # also mark the chain KMC_ERR_INVALID)
    rng = np.random.Generator(np.random.PCG64(1))
    L = float(np.sqrt(100 / workloads.DENSITY))
    net = workloads.make_network(rng, 100, 10, L, L, workloads.perimeter_electrodes(L, 65),
                                 voltages=np.zeros(65), I_0=50.0, cells=40)
    spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
    with pytest.raises(ValueError, match="at most 64 electrodes"):
        Batch([spec], [0], [1.0], [net.E_constant()], [net.electrodes[:, 3]], [net.occupation.astype(np.uint8)],
              [10], lanes=128)


def test_run_batch_host_bins_ragged_batches_like_python_batch(engine_lib):
    """A ragged batch (networks of 10..200 acceptors, 4..12 electrodes, own
    kT and hop budgets) through kmc_run_batch_host: the host path bins the
    chains by size class (its own lanes per class, one launch per class, as
    the reference's parallelSimulations takes ragged batches, goSimulation/
    simulationWrapper.go:285-309) and gives the Python Batch's results bit
    for bit."""
    import ctypes as C
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300._native import lib, check
    from kmc_dn_gb300.engine import Batch, TableSpec, default_lanes
    nets = workloads.uneven_batch(40, seed=11, hops_range=(2000, 6000))
    nc = len(nets)
    assert len({default_lanes(net.S) for net, _ in nets}) >= 3        # at least three size classes
    hops = np.array([h for _, h in nets], np.int64)
    gN = np.array([net.N for net, _ in nets], np.int32)
    gP = np.array([net.P for net, _ in nets], np.int32)
    S = gN + gP
    goff = np.concatenate([[0], np.cumsum(S.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    dist = np.concatenate([net.distances.ravel() for net, _ in nets])
    tc = np.concatenate([net.transitions_constant.ravel() for net, _ in nets])
    ec = np.concatenate([net.E_constant() for net, _ in nets])
    se = np.concatenate([net.site_energies() for net, _ in nets])
    occ = np.concatenate([net.occupation.astype(np.uint8) for net, _ in nets])
    kT = np.array([net.kT for net, _ in nets])
    t_out = np.zeros(nc)
    eo = np.zeros(int(gP.sum()), np.int64)
    st = np.zeros(nc, np.int32)
    seed = 4242
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(lib().kmc_run_batch_host(nc, p(gN), p(gP), p(np.array([n.nu for n, _ in nets])),
                                   p(np.array([n.I_0 for n, _ in nets])), p(np.array([n.R for n, _ in nets])),
                                   p(goff), p(dist), p(tc), nc, p(np.arange(nc, dtype=np.int32)), p(kT), p(ec),
                                   p(se), p(occ), p(hops), seed, 0, p(t_out), p(eo), p(st)))
    specs = [TableSpec(n.N, n.P, n.nu, n.I_0, n.R, n.distances, n.transitions_constant) for n, _ in nets]
    b = Batch(specs, np.arange(nc), kT, [n.E_constant() for n, _ in nets], [n.electrodes[:, 3] for n, _ in nets],
              [n.occupation.astype(np.uint8) for n, _ in nets], hops, seed=seed)
    assert len(b._bins) >= 3
    r = b.run().results()
    np.testing.assert_array_equal(st, 0)
    np.testing.assert_array_equal(t_out, r["time"])
    np.testing.assert_array_equal(eo, np.concatenate(r["electrode_occupation"]))
    np.testing.assert_array_equal(occ.astype(bool), np.concatenate(r["occupation"]))


@pytest.mark.parametrize("pair_mode", ["table", "positions"])
def test_persistent_launch_gives_the_static_launch_results(engine_lib, pair_mode):
    """The persistent launch (resident blocks claiming work items with an
    atomic counter) runs every chain exactly as the one-item-per-warp launch
    does: bit-identical results on a ragged batch with warp and block groups,
    also when the run is split into several launches."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    nets = workloads.uneven_batch(600, seed=21, hops_range=(1000, 8000))
    hops = np.array([h for _, h in nets], np.int64)
    specs = [TableSpec.from_network(n) if pair_mode == "positions" else
             TableSpec(n.N, n.P, n.nu, n.I_0, n.R, n.distances, n.transitions_constant) for n, _ in nets]

    def run(persistent, seg=None):
        b = Batch(specs, np.arange(len(nets)), [n.kT for n, _ in nets], [n.E_constant() for n, _ in nets],
                  [n.electrodes[:, 3] for n, _ in nets], [n.occupation.astype(np.uint8) for n, _ in nets], hops,
                  seed=13, pair_mode=pair_mode, lanes=lambda S: 16 if S <= 48 else 32 if S <= 128 else 128,
                  persistent=persistent, record=2)
        if seg is None:
            b.run()
        else:
            for _ in range(int(np.ceil(hops.max() / seg))):
                b.launch(seg)
        return b.results()
    a, p, q = run(False), run(True), run(True, seg=2048)
    assert np.all(a["status"] == 0)
    for r in (p, q):
        np.testing.assert_array_equal(a["time"], r["time"])
        np.testing.assert_array_equal(a["hops_done"], r["hops_done"])
        for k in ("electrode_occupation", "occupation", "traffic"):
            for x, y in zip(a[k], r[k]):
                np.testing.assert_array_equal(x, y)
    for x, y in zip(a["occ_time"], p["occ_time"]):
        np.testing.assert_array_equal(x, y)
    # a split run closes each occupied site's interval at every launch end and
    # adds the pieces: the same sum in another order, equal to rounding
    for x, y in zip(a["occ_time"], q["occ_time"]):
        np.testing.assert_allclose(x, y, rtol=1e-14, atol=0)


def test_f64_batch_launch_equals_single_chain_runs(engine_lib):
    """kmc_simulate_f64_batch (one block per chain, one launch) runs each
    chain exactly as kmc_simulate_f64 does with the same seed: times,
    electrode counts, final states, recorded occupancy times and flux
    integrals bit for bit, for networks of different sizes in one launch."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import simulate_f64, simulate_f64_many
    nets = [n for n, _ in workloads.uneven_batch(6, seed=8, hops_range=(1000, 1000))]
    nets.append(workloads.plain_network(1))
    chains = [dict(N=n.N, P=n.P, nu=n.nu, kT=n.kT, I_0=n.I_0, R=n.R, occupation=n.occupation.astype(np.uint8),
                   distances=n.distances, E_constant=n.E_constant(), site_energies=n.site_energies(),
                   transitions_constant=n.transitions_constant) for n in nets]
    seeds = [101 + 7 * k for k in range(len(nets))]
    hops = 1500
    t, eo, st, oit, fx = simulate_f64_many(chains, hops, seeds, record=True, flux=True)
    np.testing.assert_array_equal(st, 0)
    for k, (n, ch) in enumerate(zip(nets, chains)):
        r = simulate_f64(n.N, n.P, n.nu, n.kT, n.I_0, n.R, ch["occupation"], n.distances, ch["E_constant"],
                         ch["site_energies"], n.transitions_constant, hops, record=True, seed=seeds[k], flux=True)
        assert r["time"] == t[k]
        np.testing.assert_array_equal(r["electrode_occupation"], eo[k])
        np.testing.assert_array_equal(r["occupations_in_time"], oit[k])
        np.testing.assert_array_equal(r["flux_time"], fx[k])


def test_uniform_temperature_table_guards_its_chains(engine_lib):
    """A launch whose chains share one kT stages its pair table with the
    temperature folded in; a chain whose kT differs from the launch's
    uniform_kT stops with KMC_ERR_INVALID instead of using that table."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300._native import KMC_ERR_INVALID
    from kmc_dn_gb300.engine import Batch, TableSpec
    n = workloads.plain_network(0)
    spec = TableSpec(n.N, n.P, n.nu, n.I_0, n.R, n.distances, n.transitions_constant)
    b = Batch([spec], [0, 0], [1.0, 1.0], [n.E_constant()] * 2, [n.electrodes[:, 3]] * 2,
              [n.occupation.astype(np.uint8)] * 2, [2048, 2048], lanes=16)
    assert b.uniform_kT == 1.0
    b.uniform_kT = 0.75                     # as if the table were staged for another kT
    r = b.run().results()
    assert np.all(r["status"] == KMC_ERR_INVALID) and np.all(r["hops_done"] == 0)


def test_preload_kernels_is_idempotent_and_launches_follow(engine_lib):
    """kmc_preload_kernels loads every kernel of the library on the current
    device (a lazily loaded kernel would wait for the size bins already
    running); calling it again is a no-op, and launches work after it."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    assert engine_lib.kmc_preload_kernels() == 0
    assert engine_lib.kmc_preload_kernels() == 0
    net = workloads.plain_network(1)
    spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
    b = Batch([spec], np.zeros(4, np.int32), np.full(4, net.kT), np.tile(net.E_constant(), (4, 1)),
              np.tile(net.electrodes[:, 3], (4, 1)), np.tile(net.occupation.astype(np.uint8), (4, 1)),
              np.full(4, 2048), seed=3)
    r = b.run().results()
    assert np.all(r["status"] == 0) and np.all(r["hops_done"] == 2048)
