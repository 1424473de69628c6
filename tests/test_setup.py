"""Set-up numerics against the reference's own fixtures (thesis_indrek/tests
.kmc files, copied to tests/golden/fixtures_*.npz by make_golden.py)."""
import numpy as np
import pytest

from conftest import golden_files, load_golden
from kmc_dn_gb300 import geometry as geo
from kmc_dn_gb300.laplace import default_cells, solve_basis_fields

FIXTURES = golden_files("fixtures_*.npz")


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: p.split("fixtures_")[-1][:-4])
def test_eV_constant_matches_fenics(path):
    """FD basis fields + P1 interpolation reproduce the FEniCS potential at
    every acceptor (boundary-segment ends and the diagonal orientation
    included)."""
    f = load_golden(path)
    worst = 0.0
    for k in range(len(f["N"])):
        xdim, ydim, res = float(f["xdim"][k]), float(f["ydim"][k]), float(f["res"][k])
        el = f["electrodes"][k]
        bf = solve_basis_fields(xdim, ydim, el[:, :2], default_cells(xdim, res), default_cells(ydim, res))
        ev = bf.sample(f["acceptors"][k][:, :2])
        V = el[:, 3] @ ev[:-1] + float(f["mu"][k]) * ev[-1]
        err = np.max(np.abs(V - f["eV_constant"][k])) / np.max(np.abs(f["eV_constant"][k]))
        worst = max(worst, err)
    assert worst < 1e-11, worst


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: p.split("fixtures_")[-1][:-4])
def test_tables_match_fixture(path):
    f = load_golden(path)
    for k in range(len(f["N"])):
        acc, el = f["acceptors"][k], f["electrodes"][k]
        d = geo.site_distances(acc, el)
        np.testing.assert_array_equal(d, f["distances"][k])
        tc = geo.transitions_constant(d, float(f["nu"][k]), float(f["ab"][k]))
        np.testing.assert_allclose(tc, f["transitions_constant"][k], rtol=1e-15, atol=1e-300)
        comp = geo.compensation(acc, f["donors"][k], float(f["I_0"][k]), float(f["R"][k]))
        np.testing.assert_allclose(comp, f["comp_constant"][k], rtol=1e-13)
        R, dim = geo.dimensionless_R(int(f["N"][k]), float(f["xdim"][k]), float(f["ydim"][k]),
                                     float(f["zdim"][k]))
        assert dim == 2 and R == float(f["R"][k])


def test_default_cells_floor_division():
    assert default_cells(1.0, 0.01) == 99
    assert default_cells(20.0, 0.2) == 99


def test_1d_basis_is_linear():
    bf = solve_basis_fields(1.0, 0.0, np.array([[0.0, 0.0], [1.0, 0.0]]), 100)
    x = np.array([[0.25, 0, 0], [0.5, 0, 0]])
    v = bf.sample(x)
    np.testing.assert_allclose(v[0], [0.75, 0.5])
    np.testing.assert_allclose(v[1], [0.25, 0.5])
    np.testing.assert_allclose(v[2], [0.0, 0.0])


def test_superposition_linearity():
    from kmc_dn_gb300 import workloads
    n = workloads.plain_network(5)
    V1, V2 = np.linspace(-1, 1, 8), np.cos(np.arange(8))
    np.testing.assert_allclose(n.eV(V1 + 2 * V2), n.eV(V1) + 2 * n.eV(V2), rtol=1e-12, atol=1e-12)


def test_total_energy_detailed_balance():
    """dE of every allowed hop equals the change of total_energy (with the
    constant site term that includes compensation) -- the identity behind
    the Boltzmann checks."""
    from kmc_dn_gb300 import workloads
    n = workloads.plain_network(6)
    N, P = n.N, n.P
    Ec = n.E_constant(np.zeros(P))
    IR = n.I_0 * n.R
    occ = n.occupation.copy()
    E = Ec - IR * np.array([sum(1 / n.distances[i, j] for j in range(N) if j != i and not occ[j])
                            for i in range(N)])
    H0 = geo.total_energy(occ, n.distances, Ec, n.I_0, n.R)
    for i in np.flatnonzero(occ)[:5]:
        for j in np.flatnonzero(~occ)[:3]:
            o2 = occ.copy(); o2[i] = False; o2[j] = True
            dE = E[j] - E[i] - IR / n.distances[i, j]
            assert abs((geo.total_energy(o2, n.distances, Ec, n.I_0, n.R) - H0) - dE) < 1e-9


@pytest.mark.gpu
def test_gpu_basis_fields_match_cpu_and_fenics(engine_lib):
    """kmc_laplace_basis (sine-transform direct solve on the device) gives the
    host FD solution, and so the reference's FEniCS potential."""
    from kmc_dn_gb300.laplace import solve_basis_fields_gpu
    f = load_golden(FIXTURES[0])
    for k in range(min(3, len(f["N"]))):
        xdim, ydim, res = float(f["xdim"][k]), float(f["ydim"][k]), float(f["res"][k])
        el = f["electrodes"][k]
        nx, ny = default_cells(xdim, res), default_cells(ydim, res)
        cpu = solve_basis_fields(xdim, ydim, el[:, :2], nx, ny)
        gpu = solve_basis_fields_gpu(xdim, ydim, el[:, :2], nx, ny)
        np.testing.assert_allclose(gpu.fields, cpu.fields, atol=1e-11, rtol=0)
        ev = gpu.sample(f["acceptors"][k][:, :2])
        V = el[:, 3] @ ev[:-1] + float(f["mu"][k]) * ev[-1]
        err = np.max(np.abs(V - f["eV_constant"][k])) / np.max(np.abs(f["eV_constant"][k]))
        assert err < 1e-11, err
    # a rectangular, anisotropic mesh too
    el = np.array([[0.0, 1.0], [3.0, 1.0], [1.5, 0.0], [1.5, 2.0]])
    cpu = solve_basis_fields(3.0, 2.0, el, 60, 45)
    gpu = solve_basis_fields_gpu(3.0, 2.0, el, 60, 45)
    np.testing.assert_allclose(gpu.fields, cpu.fields, atol=1e-11, rtol=0)


@pytest.mark.gpu
def test_gpu_p1_sampling_matches_host(engine_lib):
    import ctypes as C
    import torch
    from kmc_dn_gb300._native import lib, check
    from kmc_dn_gb300.laplace import interpolate_p1
    el = np.array([[0.0, 5.0], [20.0, 5.0], [5.0, 0.0], [5.0, 20.0]])
    bf = solve_basis_fields(20.0, 20.0, el, 100, 100)
    pts = np.random.default_rng(0).uniform(0, 20, (500, 2))
    g = torch.as_tensor(bf.fields).cuda().contiguous()
    xy = torch.as_tensor(pts).cuda().contiguous()
    out = torch.zeros(bf.fields.shape[0] * 500, dtype=torch.float64, device="cuda")
    check(lib().kmc_p1_sample(100, 100, 0.2, 0.2, bf.fields.shape[0], C.c_void_p(g.data_ptr()), 500,
                              C.c_void_p(xy.data_ptr()), C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    host = np.stack([interpolate_p1(f, bf, pts) for f in bf.fields])
    np.testing.assert_allclose(out.cpu().numpy().reshape(host.shape), host, rtol=1e-13, atol=1e-13)


def _superpose_cases():
    """The networks whose device superposition feeds the timed workloads: the
    homogeneous ensemble's network with its first voltage vectors, and the
    four serving geometries with populations of U[-1,1] vectors."""
    from kmc_dn_gb300 import workloads
    net, V = workloads.homogeneous_ensemble(64, 0)
    cases = [("homogeneous", net, V)]
    rng = np.random.default_rng(17)
    for g in workloads.serving_geometries(seed=0):
        cases.append((f"serving_N{g.N}", g, rng.uniform(-1, 1, (48, g.P))))
    return cases


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(5), ids=["homogeneous", "serving_N30", "serving_N60",
                                                "serving_N120", "serving_N240"])
def test_device_superposition_matches_host_E_constant(engine_lib, case):
    """kmc_site_energies (the device superposition that builds every timed
    chain's constant site energies and every serving request's) equals the
    host E_constant = V @ basis + mu * basis_mu + comp
    (calc_E_constant_V_comp, kmc_dopant_networks.py:865-899) rounded to FP32.

    Tolerance: the device sums the same FP64 terms in another order and
    rounds once to FP32, so each value may land one FP32 ulp away from the
    rounded host value: |dE| <= 2^-23 |E| (plus 1e-12 absolute for the FP64
    summation order near E = 0).  Electrode energies are the voltages
    rounded to FP32, exactly."""
    from kmc_dn_gb300.engine import superpose
    name, net, V = _superpose_cases()[case]
    ec, ve = superpose(net.basis, net.comp, V, net.mu, dev="cuda")
    ec = ec.cpu().numpy().reshape(V.shape[0], net.N).astype(np.float64)
    ve = ve.cpu().numpy().reshape(V.shape[0], net.P)
    host = np.stack([net.E_constant(v) for v in V])
    err = np.abs(ec - host.astype(np.float32).astype(np.float64))
    tol = 2.0 ** -23 * np.abs(host) + 1e-12
    assert np.all(err <= tol), (name, float((err / np.maximum(tol, 1e-300)).max()))
    assert np.max(np.abs(ec - host)) <= 2.0 ** -22 * np.max(np.abs(host)), name   # 2 ulp of max|E|
    np.testing.assert_array_equal(ve, V.astype(np.float32))
