"""Seeded synthetic dopant networks for the benchmark workloads and tests.

Every builder takes a seed and returns ``Network`` objects built with the
set-up restatements of ``geometry`` and ``laplace`` -- the same inputs the
reference's ``kmc_dn`` constructor produces (acceptor/donor placement,
distances, transitions_constant, E_constant = eV + compensation).  The
reference publishes no dataset for this path, so these seeded networks stand
in for its random ``kmc_dn`` instances, with the shapes and value
distributions of each workload:

* ``plain_network``        -- N=30, M=3, 20x20 box, 8 electrodes two per edge
                              at 1/3 and 2/3, V ~ U[-1,1], I_0=50 kT, ab=R,
                              101x101-vertex Laplace grid.
* ``homogeneous_ensemble`` -- that geometry with one voltage vector per chain.
* ``uneven_batch``         -- N ~ U{10..200}, M = round(0.1 N), P ~ U{4..12}
                              evenly spaced on the boundary, side scaled to the
                              same acceptor density, kT log-uniform [0.5, 5],
                              ab/R ~ U[0.5, 2], V ~ U[-2, 2], hops log-uniform.
* ``large_network``        -- N=1000, M=100, same density, 8 electrodes.
* ``serving_geometries``   -- N in {30, 60, 120, 240}, M = 0.1 N, 8 electrodes.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import geometry as geo
from .laplace import solve_basis_fields

__all__ = ["Network", "make_network", "plain_network", "homogeneous_ensemble",
           "uneven_batch", "large_network", "serving_geometries", "edge_thirds",
           "perimeter_electrodes", "DENSITY"]

DENSITY = 30 / 400.0       # acceptors per unit area of the 20x20, N=30 network


@dataclass
class Network:
    """One dopant network: positions, constants and per-geometry tables.

    ``basis`` holds the unit-voltage Laplace solutions sampled at the
    acceptors, shape (P + 1, N): rows 0..P-1 are the electrodes, row P the
    ``mu`` boundary.  ``E_constant(V)`` superposes them and adds the donor
    compensation, which is what calc_E_constant_V_comp computes after a
    FEniCS solve (kmc_dopant_networks.py:865-899)."""
    N: int
    M: int
    xdim: float
    ydim: float
    zdim: float
    acceptors: np.ndarray
    donors: np.ndarray
    electrodes: np.ndarray            # (P, 4): x, y, z, voltage
    nu: float
    kT: float
    I_0: float
    R: float
    ab: float
    mu: float
    distances: np.ndarray
    transitions_constant: np.ndarray
    comp: np.ndarray
    basis: np.ndarray
    occupation: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def P(self):
        return self.electrodes.shape[0]

    @property
    def S(self):
        return self.N + self.P

    def eV(self, voltages=None):
        v = self.electrodes[:, 3] if voltages is None else np.asarray(voltages, np.float64)
        return v @ self.basis[:-1] + self.mu * self.basis[-1]

    def E_constant(self, voltages=None):
        return self.eV(voltages) + self.comp

    def site_energies(self, voltages=None):
        """Length-S array whose electrode entries hold the electrode voltages,
        the layout the hop loops read electrode energies from."""
        v = self.electrodes[:, 3] if voltages is None else np.asarray(voltages, np.float64)
        se = np.zeros(self.S)
        se[self.N:] = v
        return se


_UNIT_BASIS = {}


def unit_square_basis(electrodes_unit, cells):
    """Basis fields of a square with electrodes at the given positions in
    unit coordinates.  The Laplace problem is scale invariant and the
    electrode segment half-width (xdim/10) scales with the side, so every
    square network with the same relative electrode layout shares them."""
    key = (tuple(map(tuple, np.round(np.asarray(electrodes_unit, np.float64), 12))), int(cells))
    bf = _UNIT_BASIS.get(key)
    if bf is None:
        bf = solve_basis_fields(1.0, 1.0, np.asarray(electrodes_unit, np.float64), cells, cells)
        _UNIT_BASIS[key] = bf
    return bf


def make_network(rng, N, M, xdim, ydim, electrodes_xy, *, voltages, I_0=50.0, a=1.0,
                 kT=1.0, nu=1.0, mu=0.0, cells=100, ab_over_R=None):
    """Build a 2D network with random acceptors/donors and the given electrodes.

    I_0 is in units of kT as in the constructor (``I_0 = I_0_arg * kT``,
    kmc_dopant_networks.py:338); ab = a*R (:361) unless ab_over_R is given.
    Square domains reuse the unit-square basis fields of their electrode
    layout."""
    R, dim = geo.dimensionless_R(N, xdim, ydim, 0)
    assert dim == 2
    acc, don = geo.place_dopants(rng, N, M, xdim, ydim, 0)
    occ = geo.place_charges(rng, N, M)
    P = len(electrodes_xy)
    el = np.zeros((P, 4))
    el[:, :2] = np.asarray(electrodes_xy, dtype=np.float64).reshape(P, 2)
    el[:, 3] = voltages
    ab = (ab_over_R if ab_over_R is not None else a) * R
    I0 = I_0 * kT
    dist = geo.site_distances(acc, el)
    tc = geo.transitions_constant(dist, nu, ab)
    comp = geo.compensation(acc, don, I0, R)
    if xdim == ydim:
        bf = unit_square_basis(el[:, :2] / xdim, cells)
        basis = bf.sample(acc[:, :2] / xdim)
    else:
        bf = solve_basis_fields(xdim, ydim, el[:, :2], cells, cells)
        basis = bf.sample(acc[:, :2])
    return Network(N=N, M=M, xdim=float(xdim), ydim=float(ydim), zdim=0.0, acceptors=acc,
                   donors=don, electrodes=el, nu=float(nu), kT=float(kT), I_0=float(I0),
                   R=float(R), ab=float(ab), mu=float(mu), distances=dist,
                   transitions_constant=tc, comp=comp, basis=basis, occupation=occ)


def edge_thirds(L):
    """8 electrodes, two per edge at 1/3 and 2/3 of the side (left, right,
    bottom, top -- the edge order of thesis_indrek/generate_tests.py:34-41)."""
    t1, t2 = L / 3, 2 * L / 3
    return [(0.0, t1), (0.0, t2), (L, t1), (L, t2), (t1, 0.0), (t2, 0.0), (t1, L), (t2, L)]


def perimeter_electrodes(L, P):
    """P electrodes evenly spaced along the perimeter at arc positions
    (k + 1/2) * 4L/P, walking bottom, right, top, left."""
    out = []
    for k in range(P):
        s = (k + 0.5) * 4 * L / P
        edge, t = int(s // L), s - L * int(s // L)
        if edge == 0:
            out.append((t, 0.0))
        elif edge == 1:
            out.append((L, t))
        elif edge == 2:
            out.append((L - t, L))
        else:
            out.append((0.0, L - t))
    return out


def plain_network(seed=0, N=30, M=3, L=20.0):
    """The single-chain FP64 workload's network (N=30, M=3, 20x20, 8 electrodes)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    V = rng.uniform(-1.0, 1.0, 8)
    return make_network(rng, N, M, L, L, edge_thirds(L), voltages=V, I_0=50.0, a=1.0)


def homogeneous_ensemble(n_chains, seed=0):
    """The plain network with an independent U[-1,1] voltage vector per chain.

    Returns (network, voltages[n_chains, 8])."""
    net = plain_network(seed)
    rng = np.random.Generator(np.random.PCG64(seed + 1_000_003))
    return net, rng.uniform(-1.0, 1.0, (n_chains, net.P))


def uneven_batch(n_chains, seed=0, hops_range=(1e4, 1e6), cells=100):
    """Heterogeneous networks: one per chain.  Returns a list of
    (network, hops) pairs."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n_chains):
        N = int(rng.integers(10, 201))
        M = int(round(0.1 * N))
        P = int(rng.integers(4, 13))
        L = float(np.sqrt(N / DENSITY))
        kT = float(np.exp(rng.uniform(np.log(0.5), np.log(5.0))))
        ab_over_R = float(rng.uniform(0.5, 2.0))
        V = rng.uniform(-2.0, 2.0, P)
        hops = int(round(np.exp(rng.uniform(np.log(hops_range[0]), np.log(hops_range[1])))))
        net = make_network(rng, N, M, L, L, perimeter_electrodes(L, P), voltages=V,
                           I_0=50.0, kT=kT, ab_over_R=ab_over_R, cells=cells)
        out.append((net, hops))
    return out


def large_network(seed=0, N=1000, M=100):
    rng = np.random.Generator(np.random.PCG64(seed))
    L = float(np.sqrt(N / DENSITY))
    V = rng.uniform(-1.0, 1.0, 8)
    return make_network(rng, N, M, L, L, edge_thirds(L), voltages=V, I_0=50.0)


def serving_geometries(seed=0, sizes=(30, 60, 120, 240)):
    out = []
    for k, N in enumerate(sizes):
        rng = np.random.Generator(np.random.PCG64(seed * 7919 + k))
        L = float(np.sqrt(N / DENSITY))
        V = np.zeros(8)
        out.append(make_network(rng, N, int(round(0.1 * N)), L, L, edge_thirds(L),
                                voltages=V, I_0=50.0))
    return out
