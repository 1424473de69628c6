"""Mean-field relaxation on the device: the Go library's ``probSimulate``
(goSimulation/probabilitySimulation.go:53-157), reached from the reference as
``kmc.go_simulation(hops=1000, goSpecificFunction="wrapperSimulateProbability")``
(dn_search.py:49-52 uses it as the cheapest first search stage).

The state is the occupation probability of every acceptor; each iteration
moves the expected charge along the expected rates and advances the time by
0.98 of the largest admissible step.  ``run`` relaxes a batch of networks in
one launch (one thread block per network, kmc_mf_run); ``simulate_probability``
takes ``callGoSimulation``'s keyword set and returns what it returns.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from ._native import KmcMfBatch, check, lib

__all__ = ["Network", "MeanFieldBatch", "run", "simulate_probability", "max_sites"]

RATES = {"f64": _native.MF_RATES_F64, "f32": _native.MF_RATES_F32}


class Network:
    """One network's inputs: sizes, constants, S x S distances and
    transition constants, N constant energies, P electrode voltages."""

    def __init__(self, N, P, nu, kT, I_0, R, distances, transitions_constant, E_constant, voltages):
        self.N, self.P = int(N), int(P)
        self.nu, self.kT, self.I_0, self.R = float(nu), float(kT), float(I_0), float(R)
        S = self.N + self.P
        self.distances = np.ascontiguousarray(distances, np.float64).reshape(S, S)
        self.transitions_constant = np.ascontiguousarray(transitions_constant, np.float64).reshape(S, S)
        self.E_constant = np.ascontiguousarray(E_constant, np.float64).reshape(self.N)
        self.voltages = np.ascontiguousarray(voltages, np.float64).reshape(self.P)


def max_sites(rates="f64"):
    """Largest network (acceptors + electrodes) one block holds."""
    return int(lib().kmc_mf_max_sites(RATES[rates]))


class MeanFieldBatch:
    """Device buffers of one batch of networks, launched with ``launch`` as
    often as wanted (each launch restarts from ``start``)."""

    def __init__(self, networks, hops, *, rates="f64", record=False, start=0.5, dev=None):
        import torch
        nets = list(networks)
        n = len(nets)
        if n == 0:
            raise ValueError("no networks")
        h = np.broadcast_to(np.asarray(hops, dtype=np.int64), (n,)).copy()
        if (h < 0).any():
            raise ValueError("hops must be >= 0")
        self.nets, self.n, self.record = nets, n, bool(record)
        self.mode = RATES[rates]
        Ns = np.array([x.N for x in nets], np.int32)
        Ps = np.array([x.P for x in nets], np.int32)
        Ss = Ns.astype(np.int64) + Ps
        lim = max_sites(rates)
        if Ss.max() > lim:
            raise ValueError(f"a network has {int(Ss.max())} sites; the {rates} kernel holds at most {lim}")
        # pair blocks, shared by identity
        pair_off = np.zeros(n, np.int64)
        blocks, seen, off = [], {}, 0
        for c, x in enumerate(nets):
            key = (id(x.distances), id(x.transitions_constant))
            if key not in seen:
                seen[key] = off
                blocks.append((x.distances, x.transitions_constant))
                off += x.distances.size
            pair_off[c] = seen[key]
        self.site_off = np.concatenate([[0], np.cumsum(Ss)[:-1]]).astype(np.int64)
        self.el_off = np.concatenate([[0], np.cumsum(Ps.astype(np.int64))[:-1]]).astype(np.int64)
        self.tr_off = np.concatenate([[0], np.cumsum(Ss * Ss)[:-1]]).astype(np.int64)
        self.S = Ss
        n_sites = int(Ss.sum())
        ec = np.zeros(n_sites)
        se = np.zeros(n_sites)
        occ = np.zeros(n_sites)
        for c, x in enumerate(nets):
            o = self.site_off[c]
            ec[o:o + x.N] = x.E_constant
            se[o + x.N:o + x.N + x.P] = x.voltages
            occ[o:o + x.N] = start
        self.dev = d = torch.device(dev if dev is not None else "cuda")
        f64, i64, i32 = torch.float64, torch.int64, torch.int32
        T = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a)).to(device=d, dtype=dt)  # noqa: E731
        self.t = t = {}
        t["N"], t["P"] = T(Ns, i32), T(Ps, i32)
        for k in ("nu", "kT", "I_0", "R"):
            t[k] = T([getattr(x, k) for x in nets], f64)
        t["pair_off"] = T(pair_off, i64)
        t["distances"] = T(np.concatenate([b[0].ravel() for b in blocks]), f64)
        t["transitions_constant"] = T(np.concatenate([b[1].ravel() for b in blocks]), f64)
        t["site_off"], t["E_constant"] = T(self.site_off, i64), T(ec, f64)
        self._se0, self._occ0 = T(se, f64), T(occ, f64)
        t["site_energies"], t["occupation"] = self._se0.clone(), self._occ0.clone()
        t["el_off"] = T(self.el_off, i64)
        t["electrode_occupation"] = torch.zeros(max(int(Ps.sum()), 1), dtype=f64, device=d)
        t["hops"] = T(h, i64)
        t["time"] = torch.zeros(n, dtype=f64, device=d)
        t["status"] = torch.zeros(n, dtype=i32, device=d)
        t["iterations_done"] = torch.zeros(n, dtype=i64, device=d)
        if record:
            t["traffic_off"] = T(self.tr_off, i64)
            t["traffic"] = torch.zeros(int((Ss * Ss).sum()), dtype=f64, device=d)
            t["average_occupation"] = torch.zeros(n_sites, dtype=f64, device=d)
        b = KmcMfBatch()
        b.n_chains, b.max_sites, b.rates, b.record = n, int(Ss.max()), self.mode, int(self.record)
        for name, _ in KmcMfBatch._fields_[4:]:
            v = t.get(name)
            setattr(b, name, v.data_ptr() if v is not None else None)
        self.b = b
        self.pairs_per_iteration = int((Ss * Ss).sum())

    def reset(self):
        """Back to the starting probabilities (the traffic and occupancy sums
        of record mode are zeroed too)."""
        t = self.t
        t["occupation"].copy_(self._occ0)
        t["site_energies"].copy_(self._se0)
        if self.record:
            t["traffic"].zero_()
            t["average_occupation"].zero_()

    def launch(self, stream=None):
        import torch
        st = stream if stream is not None else torch.cuda.current_stream(self.dev)
        check(lib().kmc_mf_run(C.byref(self.b), C.c_void_p(st.cuda_stream)))

    def results(self):
        import torch
        torch.cuda.synchronize(self.dev)
        t, nets, n = self.t, self.nets, self.n
        so, eo_off = self.site_off, self.el_off
        occ_h, se_h = t["occupation"].cpu().numpy(), t["site_energies"].cpu().numpy()
        eo_h = t["electrode_occupation"].cpu().numpy()
        out = dict(time=t["time"].cpu().numpy(), status=t["status"].cpu().numpy(),
                   iterations=t["iterations_done"].cpu().numpy(),
                   occupation=[occ_h[so[c]:so[c] + nets[c].N].copy() for c in range(n)],
                   site_energies=[se_h[so[c]:so[c] + nets[c].N].copy() for c in range(n)],
                   electrode_occupation=[eo_h[eo_off[c]:eo_off[c] + nets[c].P].copy() for c in range(n)])
        if self.record:
            tr_h, avg_h = t["traffic"].cpu().numpy(), t["average_occupation"].cpu().numpy()
            S, to = self.S, self.tr_off
            out["traffic"] = [tr_h[to[c]:to[c] + S[c] ** 2].reshape(S[c], S[c]).copy() for c in range(n)]
            out["average_occupation"] = [avg_h[so[c]:so[c] + nets[c].N].copy() for c in range(n)]
        return out


def run(networks, hops, *, rates="f64", record=False, start=0.5, dev=None, stream=None):
    """Relax every network for ``hops`` iterations (int or one per network).

    Networks that share the same ``distances`` and ``transitions_constant``
    arrays (the same objects) share one pair block on the device.  Returns a
    dict of host arrays: time[C], occupation (list of N-vectors),
    electrode_occupation (list of P-vectors), site_energies (list of
    N-vectors), status[C], iterations[C] and, with record, traffic (list of
    S x S) and average_occupation (list of N-vectors, time-weighted sums)."""
    b = MeanFieldBatch(networks, hops, rates=rates, record=record, start=start, dev=dev)
    b.launch(stream)
    return b.results()


def simulate_probability(N_acceptors, N_electrodes, nu, kT, I_0, R, time, occupation, distances,
                         E_constant, site_energies, transitions_constant, transitions=None,
                         problist=None, electrode_occupation=None, hops=1000, record=False,
                         goSpecificFunction="wrapperSimulateProbability", prune_threshold=0.0,
                         rates="f64", **_ignored):
    """Drop-in for ``callGoSimulation(..., goSpecificFunction=
    "wrapperSimulateProbability")`` (goSimulation/pythonBind.py:49-92).

    The relaxation starts from 0.5 on every acceptor
    (simulationWrapper.go:229-232).  As through the ctypes bridge, the
    returned occupation and electrode_occupation are the Go slices' values
    truncated to int (pythonBind.py:85-86); the time and, with record, the
    traffic and time-weighted occupation sums are returned as floats."""
    N, P = int(N_acceptors), int(N_electrodes)
    S = N + P
    se = np.asarray(site_energies, np.float64).reshape(S)
    net = Network(N, P, nu, kT, I_0, R, distances, transitions_constant, E_constant, se[N:])
    r = run([net], int(hops), rates=rates, record=record)
    if r["status"][0] != 0:
        raise _native.KmcError(int(r["status"][0]), "mean-field relaxation stopped: total rate zero or non-finite")
    t = float(r["time"][0])
    occ = np.array([int(x) for x in r["occupation"][0]])
    eo = np.array([int(x) for x in r["electrode_occupation"][0]])
    if not record:
        return t, occ, eo
    return t, occ, eo, r["traffic"][0], r["average_occupation"][0]
