"""Batched runs with the reference's ``parrallelSimulation`` interface.

``parrallelSimulation.addSimulation(dn, hops)`` collects networks and
``runSimulation()`` runs them all at once, appending ``(time,
electrode_occupation, current)`` to each ``dn.parrallel_results``
(goSimulation/parrallelSimulationBind.py:9-79).  The reference runs one
goroutine per network with the Go ``simulateRecordPlus`` loop starting from
each network's occupation (simulationWrapper.go:250-315); here every network
is one chain of a single batched FP32 engine run, with networks that share
their geometry tables sharing one device table.
"""
from __future__ import annotations

import numpy as np

from .engine import Batch, TableSpec

__all__ = ["parrallelSimulation", "shard_range", "replica_chains", "reduce_step"]


class parrallelSimulation:
    def __init__(self, seed=None, lanes=None):
        self.dns = []
        self.hops = []
        self.seed = seed
        self.lanes = lanes

    def addSimulation(self, dn, hops):
        dn.parrallel_results = []
        self.dns.append(dn)
        self.hops.append(int(hops))

    def runSimulation(self):
        if not self.dns:
            return
        specs, keys, chain_tab = [], {}, []
        for dn in self.dns:
            k = (id(dn.distances), id(dn.transitions_constant), dn.N, dn.P, dn.I_0, dn.R, dn.nu)
            if k not in keys:
                keys[k] = len(specs)
                specs.append(TableSpec(dn.N, dn.P, float(dn.nu), float(dn.I_0), float(dn.R),
                                       np.asarray(dn.distances, np.float64),
                                       np.asarray(dn.transitions_constant, np.float64)))
            chain_tab.append(keys[k])
        seed = self.seed if self.seed is not None else int(np.random.randint(0, 2**63 - 1, dtype=np.int64))
        b = Batch(specs, chain_tab, [float(dn.kT) for dn in self.dns],
                  [np.asarray(dn.E_constant, np.float64) for dn in self.dns],
                  [np.asarray(dn.site_energies, np.float64)[dn.N:] for dn in self.dns],
                  [np.asarray(dn.occupation).astype(np.uint8) for dn in self.dns], self.hops,
                  seed=seed, lanes=self.lanes)
        r = b.run().results()
        for i, dn in enumerate(self.dns):
            t = float(r["time"][i])
            eo = [float(x) for x in r["electrode_occupation"][i]]
            dn.parrallel_results.append((t, eo, [e / t for e in eo]))
        return r


def shard_range(n_items, rank, world):
    """Contiguous share of n_items for one rank (sizes differ by at most one)."""
    base, extra = divmod(int(n_items), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def replica_chains(rank, n_chains):
    """Replica layout over ranks (one process per GPU, weak scaling): rank r
    runs chains [r*n, (r+1)*n) of the ensemble, with those global indices as
    their random-stream ids, so no two ranks draw the same stream and the
    union over ranks is one larger ensemble.  Returns (chain_offset,
    stream_ids)."""
    off = int(rank) * int(n_chains)
    return off, np.arange(n_chains, dtype=np.int64) + off


def reduce_step(total_ms, hops, device=None):
    """Whole-job figures of a timed region across ranks: the slowest rank's
    time and the hops of all ranks (one all-reduce each; no collective runs
    inside the timed region).  Single process: returned unchanged."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(total_ms), int(hops)
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    h = torch.tensor([int(hops)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(h, op=dist.ReduceOp.SUM)
    return float(t.item()), int(h.item())
