"""Autotuner for the batched engine's launch shape.

For a size class (sites per chain) it times short runs of the engine on
synthetic chains of that size for every lanes-per-chain G (warp slices 4..32
up to 256 sites, block groups 64..512 from 48 sites) and warps per block in
{4, 8}, on the device at hand, with the class's own chain count, and keeps
the fastest (hops/s).  Results are cached per (GPU name, size class, number of
chains) in a JSON file (``KMC_DN_AUTOTUNE_CACHE`` or
``~/.cache/kmc_dn_gb300/autotune.json``), so a workload is tuned once per
machine.  ``choose`` returns a ``lanes`` callable for ``Batch`` whose
``warps`` attribute maps each picked width to its warps per block.
"""
from __future__ import annotations

import json
import os
import threading
import time

import numpy as np

__all__ = ["tune_size_class", "choose", "size_class", "cache_path", "CANDIDATE_LANES",
           "CANDIDATE_WARPS"]

CANDIDATE_LANES = (4, 8, 16, 32, 64, 128, 256, 512)
CANDIDATE_WARPS = (4, 8)
_CLASS_EDGES = (24, 48, 96, 160, 256, 512, 1024, 2048)
_LOCK = threading.Lock()


def size_class(S):
    """Upper edge of the size class that S falls in."""
    for e in _CLASS_EDGES:
        if S <= e:
            return e
    return _CLASS_EDGES[-1]


def cache_path():
    return os.environ.get("KMC_DN_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "kmc_dn_gb300", "autotune.json"))


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def _key(gpu, sc, n_chains):
    # chain counts in powers of two: occupancy is what changes with them
    return f"{gpu}|S<={sc}|C~{1 << max(0, int(np.ceil(np.log2(max(n_chains, 1)))))}"


def _candidates(S):
    """Lanes per chain worth trying for S sites: warp slices up to S=256,
    block groups from S=48 up."""
    c = [G for G in (4, 8, 16, 32) if S <= 256]
    c += [G for G in (64, 128, 256, 512) if S >= 48]
    return c


def tune_size_class(S, n_chains, hops=2048, seed=0, dev=None, verbose=False, pair_mode="table", repeats=3):
    """Time every candidate (G, warps per block) for n_chains chains of S
    sites (CUDA events around ``repeats`` launches after a warm-up launch,
    the median kept, so one slow launch does not move the pick); return the
    best as dict(G, warps_per_block, hops_per_s, hop_latency_s, table).
    hop_latency_s is the launch time per hop, the per-hop latency of a chain
    at the class's chain count."""
    import torch
    from . import workloads
    from .engine import Batch, TableSpec
    N = max(1, S - 8)
    P = S - N
    rng = np.random.Generator(np.random.PCG64(seed))
    L = float(np.sqrt(N / workloads.DENSITY))
    net = workloads.make_network(rng, N, max(0, int(round(0.1 * N))), L, L,
                                 workloads.perimeter_electrodes(L, P), voltages=rng.uniform(-1, 1, P),
                                 I_0=50.0, cells=40)
    spec = TableSpec.from_network(net) if pair_mode == "positions" else \
        TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
    from ._native import KmcError
    table = []
    for G in _candidates(S):
        for W in (CANDIDATE_WARPS if G <= 32 else (8,)):
            b = Batch([spec], np.zeros(n_chains, np.int32), np.full(n_chains, net.kT),
                      np.tile(net.E_constant(), (n_chains, 1)), np.tile(net.electrodes[:, 3], (n_chains, 1)),
                      np.tile(net.occupation.astype(np.uint8), (n_chains, 1)), np.full(n_chains, 2 * hops),
                      seed=seed, lanes=G, warps_per_block=W, dev=dev, pair_mode=pair_mode)
            try:
                b.launch(1024)
            except KmcError:            # the shape does not fit (shared memory): not a candidate
                continue
            ts = []
            for _ in range(repeats):
                b.hops_done.zero_()          # each timed launch runs the same hops again
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                b.launch(hops)
                e1.record()
                e1.synchronize()
                ts.append(e0.elapsed_time(e1) * 1e-3)
            t = float(np.median(ts))
            rate = n_chains * hops / t
            table.append((G, W, rate, t / hops))
            if verbose:
                print(f"S={S} C={n_chains} G={G} W={W}: {rate:.3e} hops/s, {t / hops * 1e6:.2f} us/hop")
    G, W, rate, lat = max(table, key=lambda r: r[2])
    return dict(G=int(G), warps_per_block=int(W), hops_per_s=float(rate), hop_latency_s=float(lat),
                table=[list(map(float, r)) for r in table])


def choose(S_values, n_chains=None, dev=None, tune=True, pair_mode="table", max_tune_chains=8192):
    """Per-size-class lanes for a workload: a callable S -> G.  Each size
    class is tuned with its own chain count (from S_values, capped at
    max_tune_chains), or n_chains when given; results are cached."""
    import torch
    gpu = torch.cuda.get_device_name(dev) if torch.cuda.is_available() else "none"
    S_values = np.atleast_1d(np.asarray(S_values, dtype=np.int64))
    classes, counts = np.unique([size_class(int(s)) for s in S_values], return_counts=True)
    with _LOCK:
        cache = _load()
        picked = {}
        for sc, cnt in zip(classes.tolist(), counts.tolist()):
            nc = int(min(n_chains if n_chains else cnt, max_tune_chains))
            k = _key(gpu, sc, nc) + f"|{pair_mode}"
            if k not in cache and tune:
                cache[k] = tune_size_class(sc, nc, dev=dev, pair_mode=pair_mode)
                _save(cache)
            picked[sc] = (cache[k]["G"], cache[k].get("warps_per_block", 4)) if k in cache else None
    from .engine import default_lanes

    def lanes(S):
        g = picked.get(size_class(S))
        return g[0] if g else default_lanes(S)
    # warps per block for each picked width (Batch(warps_per_block=...))
    warps = {}
    for g in picked.values():
        if g and g[0] <= 32:
            warps[g[0]] = max(warps.get(g[0], 0), g[1])
    lanes.picked = {sc: (g[0] if g else None) for sc, g in picked.items()}
    lanes.warps = warps
    return lanes
