"""The kmc_dn-compatible class: constructor/set-up on the CPU, simulation
calls on the GPU."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from kmc_dn_gb300.kmc_dn import kmc_dn


def fixture_dn(k=0, sub="rnd_min_max"):
    f = load_golden(os.path.join(GOLDEN, f"fixtures_{sub}.npz"))
    dn = kmc_dn(int(f["N"][k]), int(f["M"][k]), float(f["xdim"][k]), float(f["ydim"][k]), 0,
                electrodes=f["electrodes"][k], acceptors=f["acceptors"][k], donors=f["donors"][k])
    return dn, {key: f[key][k] for key in f}


def test_constructor_reproduces_fixture_setup():
    dn, f = fixture_dn(3)
    assert dn.R == f["R"] and abs(dn.ab - f["ab"]) < 1e-15
    np.testing.assert_array_equal(dn.distances, f["distances"])
    np.testing.assert_allclose(dn.transitions_constant, f["transitions_constant"], rtol=1e-15, atol=1e-300)
    np.testing.assert_allclose(dn.eV_constant, f["eV_constant"], rtol=1e-11, atol=1e-9)
    np.testing.assert_allclose(dn.E_constant, f["E_constant"], rtol=1e-11, atol=1e-9)
    np.testing.assert_array_equal(dn.site_energies[dn.N:], f["electrodes"][:, 3])


def test_update_V_is_superposition():
    dn, f = fixture_dn(1)
    e0 = dn.E_constant.copy()
    dn.electrodes[:, 3] *= 2
    dn.update_V()
    np.testing.assert_allclose(dn.eV_constant, 2 * f["eV_constant"], rtol=1e-10, atol=1e-8)
    assert not np.allclose(dn.E_constant, e0)


def test_random_construction_and_save_load_roundtrip(tmp_path):
    el = np.array([[0, 5, 0, 1.0], [20, 5, 0, -1.0], [5, 0, 0, 0.5], [5, 20, 0, 0.0]])
    dn = kmc_dn(30, 3, 20, 20, 0, electrodes=el, I_0=50, a=1.0, seed=4)
    assert dn.occupation.sum() == 27 and dn.acceptors.shape == (30, 3)
    p = tmp_path / "x.kmc"
    dn.saveSelf(str(p))
    dn2 = kmc_dn(30, 3, 20, 20, 0, electrodes=el, I_0=50, a=1.0, seed=99)
    dn2.loadSelf(str(p))
    np.testing.assert_array_equal(dn2.acceptors, dn.acceptors)
    np.testing.assert_allclose(dn2.E_constant, dn.E_constant, rtol=1e-12)


def test_restricted_reader_rejects_foreign_globals(tmp_path):
    import pickle
    from kmc_dn_gb300.fixtures import read_kmc
    p = tmp_path / "bad.kmc"
    with open(p, "wb") as fh:
        pickle.dump({"x": os.getcwd}, fh)
    with pytest.raises(pickle.UnpicklingError):
        read_kmc(str(p))


def test_1d_network_setup():
    el = np.array([[0.0, 0, 0, 1.0], [1.0, 0, 0, 0.0]])
    dn = kmc_dn(1, 0, 1, 0, 0, electrodes=el, acceptors=np.array([[0.5, 0, 0]]), donors=np.zeros((0, 3)))
    assert dn.dim == 1
    np.testing.assert_allclose(dn.eV_constant, [0.5])


@pytest.mark.gpu
def test_cuda_simulation_outputs(engine_lib):
    dn, f = fixture_dn(0)
    occ0 = dn.occupation.copy()
    dn.cuda_simulation(hops=20000, seed=3)
    assert dn.time > 0 and dn.current.shape == (dn.P,)
    assert dn.electrode_occupation.dtype.kind == "i"
    # holes are conserved up to what the electrodes absorbed
    assert dn.occupation.sum() - occ0.sum() == -int(dn.electrode_occupation.sum())
    dn.cuda_simulation(hops=5000, record=True, seed=4)
    assert abs(sum(dn.traffic.ravel()) - 5000) < 1e-9
    assert len(dn.average_occupation) == dn.N and 0 <= min(dn.average_occupation) <= max(dn.average_occupation) <= 1 + 1e-9


@pytest.mark.gpu
def test_python_and_go_simulation_semantics(engine_lib):
    dn, f = fixture_dn(2)
    occ0 = dn.occupation.copy()
    dn.go_simulation(hops=10000, seed=5)
    # the Go path starts empty and hands the caller's occupation back unchanged
    np.testing.assert_array_equal(dn.occupation, occ0.astype(int))
    assert dn.electrode_occupation.sum() < 0      # holes entered the empty network
    dn.go_simulation(hops=4000, record=True, seed=6)
    np.testing.assert_allclose(dn.traffic, -dn.traffic.T)   # net traffic convention
    dn.occupation = occ0.copy()
    dn.python_simulation(hops=3000, seed=7)
    assert dn.time > 0
    dn.occupation = occ0.copy()
    dn.cuda_simulation(hops=3000, prehops=1000, seed=8)
    assert dn.time > 0


@pytest.mark.gpu
def test_current_statistics_match_fixture(engine_lib):
    """Currents on a reference fixture agree with its stored mean/sigma
    (5 reference runs of ~1e6 hops) within MC error."""
    dn, f = fixture_dn(0)
    from kmc_dn_gb300.engine import Batch, TableSpec
    reps, hops = 64, 1_000_000
    spec = TableSpec(dn.N, dn.P, dn.nu, dn.I_0, dn.R, dn.distances, dn.transitions_constant)
    b = Batch([spec], [0] * reps, [1.0] * reps, [dn.E_constant] * reps, [dn.electrodes[:, 3]] * reps,
              [np.zeros(dn.N, np.uint8)] * reps, [hops] * reps, seed=17, lanes=8)
    r = b.run().results()
    cur = np.array([e / t for e, t in zip(r["electrode_occupation"], r["time"])])
    mean, sem = cur.mean(0), cur.std(0, ddof=1) / np.sqrt(reps)
    ref_mean, ref_sd = f["mean_currents"], f["stddev_currents"]
    sig = np.sqrt(sem ** 2 + ref_sd ** 2 / 5) + 1e-30
    z = np.abs(mean - ref_mean) / sig
    assert np.all(z < 4.0), z


@pytest.mark.gpu
def test_go_simulation_probability_on_the_class(engine_lib):
    """dn_search's first stage: kmc.go_simulation(hops=1000,
    goSpecificFunction="wrapperSimulateProbability") (dn_search.py:49-52),
    with the bridge's int-truncated counts and current = counts / time."""
    import oracle as O
    dn, f = fixture_dn(1)
    dn.go_simulation(hops=1000, goSpecificFunction="wrapperSimulateProbability", record=True)
    ref = O.prob_simulate(dn.N, dn.P, dn.nu, dn.kT, dn.I_0, dn.R, np.full(dn.N, 0.5), dn.distances,
                          dn.E_constant, dn.site_energies, dn.transitions_constant, 1000, record=True)
    np.testing.assert_allclose(dn.time, ref["time"], rtol=1e-9)
    assert dn.electrode_occupation.dtype.kind == "i"
    np.testing.assert_allclose(dn.current, dn.electrode_occupation / dn.time)
    np.testing.assert_allclose(dn.average_occupation, ref["average_occupation"] / ref["time"], rtol=1e-9)
