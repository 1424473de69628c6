"""Pin the oracle: the C restatement of the numba hop loop must reproduce the
hop sequences that the reference's own function produced on the same replay
stream (tests/golden/replay_*.npz, made by tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import golden_files, load_golden
from kmc_dn_gb300.rng import replay_uniforms

REPLAYS = golden_files("replay_*.npz")


def run_oracle(o, g, hops=None):
    hops = int(g["hops"]) if hops is None else hops
    u = replay_uniforms(int(g["seed"]), 2 * hops)
    return o.numba_replay(int(g["N"]), int(g["P"]), float(g["nu"]), float(g["kT"]), float(g["I_0"]),
                          float(g["R"]), g["occupation"], g["distances"], g["E_constant"],
                          g["site_energies"], g["transitions_constant"], u, hops=hops, record=True)


def test_golden_present():
    assert len(REPLAYS) >= 5, "golden replay vectors missing: run tests/golden/make_golden.py"


@pytest.mark.parametrize("path", REPLAYS, ids=lambda p: p.split("replay_")[-1][:-4])
def test_oracle_matches_reference_replay(oracle_mod, path):
    g = load_golden(path)
    r = run_oracle(oracle_mod, g)
    # bit-exact hop sequence, electrode counts and final state
    np.testing.assert_array_equal(r["hop_log"], g["hop_log"].astype(np.int32))
    np.testing.assert_array_equal(r["electrode_occupation"], g["final_electrode_occupation"])
    np.testing.assert_array_equal(r["occupation"], g["final_occupation"])
    np.testing.assert_array_equal(r["traffic"], g["traffic"])
    # clock: same formula and order; libm log may differ by an ulp
    assert abs(r["time"] - float(g["time"])) <= 1e-12 * abs(float(g["time"]))
    np.testing.assert_allclose(r["occupations_in_time"], g["occupations_in_time"], rtol=1e-12, atol=0)
    if len(g["time_ckpt"]):
        every = len(r["hop_times"]) // len(g["time_ckpt"])
        ck = np.cumsum(r["hop_times"])[every - 1::every]
        np.testing.assert_allclose(ck, g["time_ckpt"], rtol=1e-12)


def test_pure_python_restatement_agrees(oracle_mod):
    """A second, independent (pure Python) restatement agrees with the C one."""
    g = load_golden([p for p in REPLAYS if "set_N1" in p or "closed" in p][0])
    hops = 300
    u = replay_uniforms(int(g["seed"]), 2 * hops)
    log, t = oracle_mod.numba_replay_py(int(g["N"]), int(g["P"]), float(g["nu"]), float(g["kT"]),
                                        float(g["I_0"]), float(g["R"]), g["occupation"], g["distances"],
                                        g["E_constant"], g["site_energies"], g["transitions_constant"], u)
    np.testing.assert_array_equal(log, g["hop_log"][:hops].astype(np.int32))
    r = run_oracle(oracle_mod, g, hops)
    assert abs(r["time"] - t) <= 1e-12 * abs(t)


def _current_z(oracle_mod, g, go_kT, hops=20000, reps=8):
    """z-scores of the electrode-current differences between the FP32 Go-path
    restatement (at temperature go_kT) and the FP64 numba restatement."""
    N, P = int(g["N"]), int(g["P"])
    cur_go, cur_nb = [], []
    for s in range(reps):
        r = oracle_mod.go_simulate(N, P, float(g["nu"]), go_kT, float(g["I_0"]), float(g["R"]),
                                   g["occupation"], g["distances"], g["E_constant"], g["site_energies"],
                                   g["transitions_constant"], hops, seed=1000 + s)
        cur_go.append(r["electrode_occupation"] / r["time"])
        u = replay_uniforms(5000 + s, 2 * hops)
        q = oracle_mod.numba_replay(N, P, float(g["nu"]), float(g["kT"]), float(g["I_0"]), float(g["R"]),
                                    g["occupation"], g["distances"], g["E_constant"], g["site_energies"],
                                    g["transitions_constant"], u, record=False)
        cur_nb.append(q["electrode_occupation"] / q["time"])
    a, b = np.array(cur_go), np.array(cur_nb)
    sig = np.sqrt(a.var(0, ddof=1) / reps + b.var(0, ddof=1) / reps) + 1e-12
    return np.abs(a.mean(0) - b.mean(0)) / sig


def test_go_restatement_statistics(oracle_mod):
    """The FP32 Go-path restatement agrees with the FP64 numba restatement in
    distribution: electrode currents over independent seeds within 4.5 sigma."""
    g = load_golden([p for p in REPLAYS if "plain" in p][0])
    z = _current_z(oracle_mod, g, float(g["kT"]))
    assert np.all(z < 4.5), z


def test_current_comparison_detects_a_planted_bias(oracle_mod):
    """The same z statistic flags a planted mistake: the Go-path restatement
    run at twice the temperature gives currents the comparison rejects."""
    g = load_golden([p for p in REPLAYS if "plain" in p][0])
    z = _current_z(oracle_mod, g, 2.0 * float(g["kT"]))
    assert np.any(z > 4.5), z


def test_golden_pin_detects_planted_mistakes(oracle_mod):
    """The golden comparison is not vacuous: mistakes planted in the oracle's
    inputs on the CPU (uniforms consumed event-then-clock instead of
    clock-then-event, a 0.1 % temperature error, two acceptors' distance rows
    exchanged) each change the replayed hop sequence."""
    g = load_golden([p for p in REPLAYS if "plain" in p][0])
    N, P = int(g["N"]), int(g["P"])
    hops = 20000
    u = replay_uniforms(int(g["seed"]), 2 * hops)
    want = g["hop_log"][:hops].astype(np.int32)

    def replay(u_, kT=float(g["kT"]), d=g["distances"]):
        r = oracle_mod.numba_replay(N, P, float(g["nu"]), kT, float(g["I_0"]), float(g["R"]), g["occupation"],
                                    d, g["E_constant"], g["site_energies"], g["transitions_constant"], u_,
                                    hops=hops, record=False)
        return r["hop_log"]

    np.testing.assert_array_equal(replay(u), want)                  # the unplanted oracle agrees
    swapped = u.reshape(-1, 2)[:, ::-1].reshape(-1).copy()
    assert not np.array_equal(replay(swapped), want)
    assert not np.array_equal(replay(u, kT=float(g["kT"]) * 1.001), want)
    d = np.array(g["distances"], np.float64).reshape(N + P, N + P).copy()
    d[[0, 1]] = d[[1, 0]]
    d[:, [0, 1]] = d[:, [1, 0]]
    assert not np.array_equal(replay(u, d=d), want)
