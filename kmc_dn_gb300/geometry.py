"""Per-geometry constants of a dopant network (host set-up, FP64).

These are the inputs the hop loop consumes; each function restates one
set-up step of the reference with the same floating-point expression order,
so that tables built here equal the reference's to the last bit when the
positions are equal:

* ``dimensionless_R``      -- R from the acceptor density, kmc_dopant_networks.py:349-358
* ``place_dopants``        -- place_dopants_random, kmc_dopant_networks.py:621-639
* ``place_charges``        -- place_charges_random, kmc_dopant_networks.py:641-655
* ``site_distances``       -- calc_distances / dist, kmc_dopant_networks.py:657-695, :1003-1006
* ``transitions_constant`` -- calc_transitions_constant, kmc_dopant_networks.py:824-830
* ``compensation``         -- donor term of calc_E_constant_V_comp, kmc_dopant_networks.py:893-895

Random placement takes a ``numpy.random.Generator`` so that every workload
is reproducible from a seed.
"""
from __future__ import annotations

import numpy as np

__all__ = ["dimensionless_R", "place_dopants", "place_charges", "site_distances",
           "transitions_constant", "compensation", "total_energy"]


def dimensionless_R(N, xdim, ydim, zdim):
    """Average acceptor spacing R = density**(-1/dim) and the dimension."""
    if ydim == 0 and zdim == 0:
        return (N / xdim) ** (-1), 1
    if zdim == 0:
        return (N / (xdim * ydim)) ** (-1 / 2), 2
    return (N / (xdim * ydim * zdim)) ** (-1 / 3), 3


def place_dopants(rng, N, M, xdim, ydim, zdim):
    """Uniform acceptor (N, 3) and donor (M, 3) positions in the box."""
    acc = rng.random((N, 3))
    don = rng.random((M, 3))
    for a in (acc, don):
        a[:, 0] *= xdim
        a[:, 1] *= ydim
        a[:, 2] *= zdim
    return acc, don


def place_charges(rng, N, M):
    """N - M holes on distinct random acceptors (rejection sampling as in the
    reference)."""
    occ = np.zeros(N, dtype=bool)
    placed = 0
    while placed < N - M:
        trial = int(rng.integers(N))
        if not occ[trial]:
            occ[trial] = True
            placed += 1
    return occ


def site_distances(acceptors, electrodes):
    """(S, S) Euclidean distances over sites ordered acceptors then electrodes.

    The sum is evaluated as ``(dx**2 + dy**2) + dz**2`` like ``kmc_dn.dist``;
    the diagonal is 0."""
    acc = np.asarray(acceptors, dtype=np.float64).reshape(-1, 3)
    el = np.asarray(electrodes, dtype=np.float64)
    el = el.reshape(-1, el.shape[-1] if el.ndim == 2 else 4)[:, :3]
    pos = np.concatenate([acc, el], axis=0)
    d = pos[:, None, :] - pos[None, :, :]
    out = np.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2 + d[..., 2] ** 2)
    np.fill_diagonal(out, 0.0)
    return out


def transitions_constant(distances, nu, ab):
    """nu*exp(-2 d/ab) with the identity subtracted (diagonal = nu - 1)."""
    tc = nu * np.exp(-2 * distances / ab)
    tc -= np.eye(distances.shape[0])
    return tc


def compensation(acceptors, donors, I_0, R):
    """I_0*R * sum_k 1/|r_i - d_k| for every acceptor (Python ``sum`` order)."""
    acc = np.asarray(acceptors, dtype=np.float64).reshape(-1, 3)
    don = np.asarray(donors, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(acc.shape[0])
    if don.shape[0] == 0:
        return out
    d = acc[:, None, :] - don[None, :, :]
    inv = 1 / np.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2 + d[..., 2] ** 2)
    s = np.zeros(acc.shape[0])
    for k in range(don.shape[0]):        # left-to-right like sum(generator)
        s = s + inv[:, k]
    return I_0 * R * s


def total_energy(occupation, distances, E_site_constant, I_0, R):
    """Hamiltonian of one occupation state, restating kmc_dn.total_energy
    (kmc_dopant_networks.py:982-1001) with the constant site term passed in:
    H = I_0 R sum_{i<j both empty} 1/d_ij - sum_{i empty} E_i.

    The reference passes eV_constant (it omits donor compensation, its own
    TODO); passing E_constant (with compensation) gives the Hamiltonian whose
    Boltzmann law the hop loop satisfies by detailed balance."""
    occ = np.asarray(occupation, dtype=bool)
    N = occ.shape[0]
    empty = ~occ
    dd = distances[:N, :N]
    iu = np.triu_indices(N, 1)
    both = empty[iu[0]] & empty[iu[1]]
    H = I_0 * R * np.sum(1.0 / dd[iu][both])
    return H - np.sum(np.asarray(E_site_constant)[empty])
