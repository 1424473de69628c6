"""``kmc_dn`` with the reference's constructor, set-up and simulation API,
whose hop loop runs on the GPU.

Mirrors the class in kmc_dopant_networks.py:165-1001.  Differences, all on
purpose:

* The potential comes from per-electrode Laplace basis fields solved once
  per electrode layout (``laplace``) instead of a FEniCS solve per voltage
  change; ``update_V`` is a superposition.  The nodal values equal the
  FEniCS P1 solution on the same mesh (checked against the reference's
  fixtures' ``eV_constant``).
* ``cuda_simulation`` is new: the batched FP32 engine (or the FP64 kernel)
  with the ``python_simulation`` semantics -- start from ``occupation``,
  leave the final state in it.
* ``python_simulation`` runs the plain FP64 kernel, which restates the numba
  loop ``_simulate_discrete_record`` (kmc_dopant_networks.py:33-135).
* ``go_simulation`` runs the FP32 engine with the Go library's semantics
  (goSimulation/simulationWrapper.go:83-147): the run starts from an empty
  acceptor occupation, ``occupation`` is returned unchanged, record mode
  counts net traffic (+1 / -1) and credits occupancy before each hop.
  ``prune_threshold`` drops pairs with ``tc <= threshold * max(tc)`` as
  ``wrapperSimulatePruned`` does (simulation.go:199-215).
* Random placement draws from ``self.rng`` (kwarg ``seed`` or ``rng``), a
  seeded ``numpy.random.Generator``, instead of the global numpy state.
"""
from __future__ import annotations

import os
import pickle

import numpy as np

from . import geometry as geo
from .laplace import default_cells, solve_basis_fields, interpolate_p1

__all__ = ["kmc_dn"]


class kmc_dn:
    def __init__(self, N, M, xdim, ydim, zdim, mu=0, I_0=100, a=0.25, **kwargs):
        if "copy_from" in kwargs:
            self.nu = kwargs["copy_from"].nu
            self.kT = kwargs["copy_from"].kT
            self.I_0 = kwargs["copy_from"].I_0
        else:
            self.nu = 1
            self.kT = 1
            self.I_0 = I_0 * self.kT
        self.time = 0
        self.mu = mu
        self.N, self.M = N, M
        self.xdim, self.ydim, self.zdim = xdim, ydim, zdim
        self.R, self.dim = geo.dimensionless_R(N, xdim, ydim, zdim)
        self.ab = a * self.R
        rng = kwargs.get("rng")
        if rng is None:
            rng = np.random.default_rng(kwargs.get("seed"))
        self.rng = rng
        if "electrodes" in kwargs:
            self.electrodes = np.array(kwargs["electrodes"], dtype=np.float64, copy=True)
            self.P = self.electrodes.shape[0]
        else:
            self.electrodes = np.zeros((0, 4))
            self.P = 0
        if "acceptors" in kwargs:
            self.acceptors = np.array(kwargs["acceptors"], dtype=np.float64, copy=True)
        if "donors" in kwargs:
            self.donors = np.array(kwargs["donors"], dtype=np.float64, copy=True)
        self.static_electrodes = (np.array(kwargs["static_electrodes"], dtype=np.float64, copy=True)
                                  if "static_electrodes" in kwargs else np.zeros((0, 4)))
        if "res" in kwargs:
            self.res = kwargs["res"]
        elif self.dim == 1:
            self.res = self.xdim / 100
        elif self.dim == 2:
            self.res = min([self.xdim, self.ydim]) / 100
        else:
            self.res = min([self.xdim, self.ydim, self.zdim]) / 100
        if kwargs.get("calc_E_constant") == "calc_E_constant_V":
            self.calc_E_constant = self.calc_E_constant_V
        else:
            self.calc_E_constant = self.calc_E_constant_V_comp
        self.initialize(dopant_placement=not hasattr(self, "acceptors"),
                        charge_placement=not hasattr(self, "donors"))

    # ------------------------------------------------------------------ setup
    def initialize(self, dopant_placement=True, charge_placement=True, distances=True, V=True,
                   E_constant=True):
        S = self.N + self.P
        self.transitions = np.zeros((S, S))
        self.transitions_constant = np.zeros((S, S))
        self.distances = np.zeros((S, S))
        self.vectors = np.zeros((S, S, 3))
        self.site_energies = np.zeros((S,))
        self.problist = np.zeros(S ** 2)
        self.occupation = np.zeros(self.N, dtype=bool)
        self.electrode_occupation = np.zeros(self.P, dtype=int)
        if dopant_placement:
            self.place_dopants_random()
        if charge_placement:
            self.place_charges_random()
        if distances:
            self.calc_distances()
            self.calc_transitions_constant()
        if V:
            self.init_V()
        if E_constant:
            self.calc_E_constant()

    def reset(self):
        """Reset time, counters and electrode_occupation; keep occupation
        (kmc_dopant_networks.py:454-471)."""
        self.time = 0
        self.old_current = 0
        self.counter = 0
        self.electrode_occupation = np.zeros(self.P, dtype=int)

    def place_dopants_random(self):
        self.acceptors, self.donors = geo.place_dopants(self.rng, self.N, self.M, self.xdim,
                                                        self.ydim, self.zdim)

    def place_charges_random(self):
        self.occupation = geo.place_charges(self.rng, self.N, self.M)

    def calc_distances(self):
        self.distances = geo.site_distances(self.acceptors, self.electrodes)
        pos = np.concatenate([self.acceptors.reshape(-1, 3), self.electrodes[:, :3]], axis=0)
        diff = pos[None, :, :] - pos[:, None, :]
        with np.errstate(invalid="ignore", divide="ignore"):
            self.vectors = np.where(self.distances[..., None] > 0,
                                    diff / self.distances[..., None], 0.0)

    def update_electrodes(self, electrodes):
        self.electrodes = electrodes
        self.P = self.electrodes.shape[0]
        self.initialize(dopant_placement=False, charge_placement=False)

    def _all_electrodes(self):
        return np.concatenate([self.electrodes.reshape(-1, 4), self.static_electrodes.reshape(-1, 4)])

    def init_V(self):
        """Solve the unit basis fields for this electrode layout (replaces
        the FEniCS set-up and solve, kmc_dopant_networks.py:706-796)."""
        el = self._all_electrodes()
        if self.dim == 1:
            self.basis_fields = solve_basis_fields(self.xdim, 0.0, el[:, :2],
                                                   default_cells(self.xdim, self.res))
        elif self.dim == 2:
            self.basis_fields = solve_basis_fields(self.xdim, self.ydim, el[:, :2],
                                                   default_cells(self.xdim, self.res),
                                                   default_cells(self.ydim, self.res))
        else:
            raise NotImplementedError("the potential is solved in 1D and 2D (as in the reference)")
        self._refresh_potential()

    def _refresh_potential(self):
        el = self._all_electrodes()
        self._nodal_V = self.basis_fields.potential(el[:, 3], self.mu)

    def V(self, x, y=None):
        """Potential at a point, P1 interpolation of the nodal solution."""
        pt = np.array([[x, 0.0 if y is None else y]])
        return float(interpolate_p1(self._nodal_V, self.basis_fields, pt)[0])

    def update_V(self):
        """Recompute the potential for the current voltages and E_constant
        (kmc_dopant_networks.py:798-821): a superposition of basis fields."""
        self._refresh_potential()
        self.calc_E_constant()

    def calc_transitions_constant(self):
        self.transitions_constant = geo.transitions_constant(self.distances, self.nu, self.ab)

    def _eV(self):
        pts = self.acceptors[:, :2] if self.dim == 2 else self.acceptors[:, :1]
        if self.dim == 1:
            pts = np.concatenate([pts, np.zeros_like(pts)], axis=1)
        return interpolate_p1(self._nodal_V, self.basis_fields, pts)

    def calc_E_constant_V(self):
        self.eV_constant = self._eV()
        self.comp_constant = np.zeros((self.N,))
        self.E_constant = self.eV_constant
        self.site_energies[self.N:] = self.electrodes[:, 3]

    def calc_E_constant_V_comp(self):
        self.eV_constant = self._eV()
        self.comp_constant = geo.compensation(self.acceptors, self.donors, self.I_0, self.R)
        self.E_constant = self.eV_constant + self.comp_constant
        self.site_energies[self.N:] = self.electrodes[:, 3]

    def load_acceptors(self, acceptors):
        self.acceptors = acceptors
        self.N = self.acceptors.shape[0]
        self.R, self.dim = geo.dimensionless_R(self.N, self.xdim, self.ydim, self.zdim)
        self.ab = self.R
        self.initialize(V=False, dopant_placement=False)

    def load_donors(self, donors):
        self.donors = donors
        self.M = self.donors.shape[0]
        self.initialize(V=False, dopant_placement=False)

    def saveSelf(self, fileName, rel_path=False):
        """Pickle the attribute dict in the reference's .kmc layout
        (kmc_dopant_networks.py:943-963)."""
        if hasattr(self, "current"):
            self.expected_current = self.current
        path = os.path.join(os.path.dirname(__file__), fileName) if rel_path else fileName
        d = {}
        for key in dir(self):
            if key.startswith("__"):
                continue
            attr = getattr(self, key)
            if isinstance(attr, (list, tuple, int, float, np.ndarray)) and not callable(attr):
                d[key] = attr
        with open(path, "wb") as f:
            pickle.dump(d, f)

    def loadSelf(self, fileName, rel_path=False):
        """Load a .kmc file (the reference's own fixtures included) with a
        restricted unpickler that only admits numpy array reconstruction."""
        from .fixtures import read_kmc
        path = os.path.join(os.path.dirname(__file__), fileName) if rel_path else fileName
        for key, val in read_kmc(path).items():
            setattr(self, key, val)
        self.initialize(dopant_placement=False, charge_placement=False)

    def total_energy(self):
        """Hamiltonian as the reference computes it (donor term omitted,
        kmc_dopant_networks.py:982-1001)."""
        return geo.total_energy(self.occupation, self.distances, self.eV_constant, self.I_0, self.R)

    @staticmethod
    def dist(ri, rj):
        return np.sqrt((ri[0] - rj[0]) ** 2 + (ri[1] - rj[1]) ** 2 + (ri[2] - rj[2]) ** 2)

    # -------------------------------------------------------------- simulation
    def _args(self):
        return {"N_acceptors": self.N, "N_electrodes": self.P, "nu": self.nu, "kT": self.kT,
                "I_0": self.I_0, "R": self.R, "time": self.time, "occupation": self.occupation,
                "distances": self.distances, "E_constant": self.E_constant,
                "site_energies": self.site_energies,
                "transitions_constant": self.transitions_constant, "transitions": self.transitions,
                "problist": self.problist, "electrode_occupation": self.electrode_occupation,
                "record": False}

    def makeSimulation(self, simulateFunction=None, preHopFunction=None, prehops=0, hops=1E5,
                       record=False, goSpecificFunction=None, prune_threshold=0.0, **engine_opts):
        """Same flow as the reference's makeSimulation (kmc_dopant_networks.py:
        544-619): reset, optional prehops (whose final occupation is kept),
        the run, then current = electrode_occupation/time."""
        from .engine import simulate_cuda
        if simulateFunction is not None:
            self.simulate_func = simulateFunction
        if preHopFunction is not None:
            self.simulate_prehop = preHopFunction
        else:
            self.simulate_prehop = simulate_cuda
        self.reset()
        args = self._args()
        if prehops != 0:
            args["hops"] = int(prehops)
            if self.simulate_prehop is simulate_cuda:
                pre_opts = {k: v for k, v in engine_opts.items() if k in ("precision", "seed", "lanes")}
                res = simulate_cuda(**args, **pre_opts)
            else:
                res = self.simulate_prehop(**args)
            self.occupation = res[1]
            self.reset()
            args["electrode_occupation"] = self.electrode_occupation
            args["occupation"] = self.occupation
        if goSpecificFunction is not None:
            args["goSpecificFunction"] = goSpecificFunction
            args["prune_threshold"] = prune_threshold
        args["hops"] = int(hops)
        args["record"] = bool(record)
        res = self.simulate_func(**args, **engine_opts)
        if record:
            (self.time, self.occupation, self.electrode_occupation, self.traffic, oit) = res[:5]
            self.average_occupation = [x / self.time for x in oit]
        else:
            self.time, self.occupation, self.electrode_occupation = res[:3]
        self.current = self.electrode_occupation / self.time

    def cuda_simulation(self, hops=1E5, prehops=0, record=False, precision="fp32", seed=None,
                        record_convention="numba", lanes=None):
        """Simulate on the GPU.  Same outputs as python_simulation:
        time, occupation (final state), electrode_occupation, current, and
        with record: traffic, average_occupation."""
        from .engine import simulate_cuda
        self.makeSimulation(simulateFunction=simulate_cuda, preHopFunction=simulate_cuda,
                            hops=hops, prehops=prehops, record=record, precision=precision,
                            seed=seed, record_convention=record_convention, lanes=lanes)

    def python_simulation(self, hops=1E5, prehops=0, record=False, seed=None):
        """The numba loop's semantics on the plain FP64 kernel."""
        self.cuda_simulation(hops=hops, prehops=prehops, record=record, precision="fp64", seed=seed)

    def go_simulation(self, hops=1E5, prehops=0, goSpecificFunction="wrapperSimulateRecord",
                      record=False, prune_threshold=0, seed=None):
        """The Go library's semantics on the FP32 engine: empty start,
        occupation returned unchanged, net traffic and pre-hop occupancy
        credit when recording."""
        from .engine import simulate_go
        self.makeSimulation(simulateFunction=simulate_go, preHopFunction=None, hops=hops,
                            prehops=prehops, goSpecificFunction=goSpecificFunction, record=record,
                            prune_threshold=prune_threshold, seed=seed)
