"""Continuous-batching request loop for voltage-search populations.

The reference's searches evaluate populations of electrode-voltage vectors
on fixed networks: ``voltage_search.parallel_simulation`` sets voltages,
re-solves the potential and queues one Go simulation per (network, test)
(voltage_search.py:138-157, dn_search.py:472-483).  Here a request is such a
population: one resident geometry, C voltage vectors, a hop budget and a
seed.  The server

* keeps every geometry resident on the device (pair tables or site
  coordinates, Laplace basis fields sampled at the acceptors, donor terms),
  so a request only ships its voltages; the constant site energies of its
  chains are superposed on the device (``kmc_site_energies``);
* admits requests in arrival order while their chain state fits the device
  memory budget, and keeps that state resident until the request is done;
* runs every admitted request in quanta of hops on a pool of CUDA streams,
  so requests that arrive while others run are started at once and their
  launches overlap on the device; the request with the least remaining work
  is launched first and short requests use the high-priority streams;
* returns per-chain currents, times and electrode counts, and records each
  request's latency (arrival to result on the host).

A request's chains draw from streams keyed by the request seed and the chain
index, and quanta start at multiples of the energy re-anchor period, so a
request's result does not depend on which requests ran beside it.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch

from . import _native
from .engine import Batch, TableSet, TableSpec, _REANCHOR, superpose

__all__ = ["Request", "Server", "latency_summary"]


@dataclass
class Request:
    geometry: int
    voltages: np.ndarray            # (C, P)
    hops: int
    seed: int
    arrival: float = 0.0            # time.perf_counter() at submission
    future: Future = field(default_factory=Future)
    done_at: Optional[float] = None
    # filled by the server
    batch: Optional[Batch] = None
    launched_hops: int = 0
    inflight: Optional[torch.cuda.Event] = None
    stream: Optional[torch.cuda.Stream] = None
    bytes: int = 0
    started: bool = False


def _request_bytes(n_chains, N, P):
    # per chain: energies (4N) + occupation (N) + electrode energies (4P) and
    # counters (8P) + time/hops/stream/status/pairs (48) + work slot (4)
    return n_chains * (5 * N + 12 * P + 52)


class Server:
    """Serve hop-loop requests on one GPU with continuous batching.

    networks:       list of workloads.Network (the resident geometries)
    quantum:        hops per launch and request (a multiple of 1024)
    mem_budget:     bytes of chain state admitted at once (default: a
                    quarter of the free device memory at start)
    n_streams:      CUDA streams launches are spread over
    pair_mode:      "positions" (tables must be those of the positions) or
                    "table"
    """

    def __init__(self, networks, *, quantum=4096, mem_budget=None, n_streams=8,
                 pair_mode="positions", lanes=None, dev=None, short_hops=20000):
        if quantum % _REANCHOR:
            raise ValueError("quantum must be a multiple of the re-anchor period (1024)")
        d = torch.device(dev if dev is not None else "cuda")
        self.dev = torch.device("cuda", d.index if d.index is not None else torch.cuda.current_device())
        self.networks = list(networks)
        self.quantum = int(quantum)
        self.pair_mode = pair_mode
        self.lanes = lanes
        self.short_hops = int(short_hops)
        free, _total = torch.cuda.mem_get_info(self.dev)
        self.mem_budget = int(mem_budget if mem_budget is not None else free // 4)
        self.mem_used = 0
        lo, hi = torch.cuda.Stream.priority_range()
        self.hi_streams = [torch.cuda.Stream(device=self.dev, priority=hi) for _ in range(max(1, n_streams // 2))]
        self.lo_streams = [torch.cuda.Stream(device=self.dev, priority=lo) for _ in range(max(1, n_streams - n_streams // 2))]
        self._rr = 0
        self.specs = [TableSpec.from_network(n) for n in self.networks]
        # one resident table set per geometry (a request names one geometry)
        self.table_sets = [TableSet([sp], pair_mode=pair_mode, dev=self.dev) for sp in self.specs]
        self.queue = deque()
        self.active = []
        self.finished = []
        self.lock = threading.Lock()
        self.cv = threading.Condition(self.lock)
        self._thread = None
        self._stop = False
        self.hops_done = 0

    # ---------------------------------------------------------------- API
    def submit(self, geometry, voltages, hops, seed):
        V = np.asarray(voltages, np.float64)
        if V.ndim != 2 or V.shape[1] != self.networks[geometry].P:
            raise ValueError("voltages must be (n_chains, P) for the geometry")
        req = Request(int(geometry), V, int(hops), int(seed), arrival=time.perf_counter())
        with self.cv:
            self.queue.append(req)
            self.cv.notify()
        return req

    def start(self):
        self._stop = False
        self._thread = threading.Thread(target=self._loop, name="kmc-serving", daemon=True)
        self._thread.start()
        return self

    def stop(self, drain=True):
        if drain:
            self.wait_idle()
        with self.cv:
            self._stop = True
            self.cv.notify()
        if self._thread is not None:
            self._thread.join()
            self._thread = None

    def wait_idle(self, timeout=None):
        t0 = time.perf_counter()
        while True:
            with self.lock:
                if not self.queue and not self.active:
                    return True
            if timeout is not None and time.perf_counter() - t0 > timeout:
                return False
            time.sleep(0.001)

    # ----------------------------------------------------------- internals
    def _admit(self):
        while self.queue:
            req = self.queue[0]
            net = self.networks[req.geometry]
            need = _request_bytes(req.voltages.shape[0], net.N, net.P)
            if self.active and self.mem_used + need > self.mem_budget:
                return
            self.queue.popleft()
            self._prepare(req, need)

    def _prepare(self, req, need):
        net = self.networks[req.geometry]
        n = req.voltages.shape[0]
        short = req.hops <= self.short_hops
        pool = self.hi_streams if short else self.lo_streams
        req.stream = pool[self._rr % len(pool)]
        self._rr += 1
        with torch.cuda.stream(req.stream):
            ec, ve = superpose(net.basis, net.comp, req.voltages, net.mu, dev=self.dev, stream=req.stream)
            req.batch = Batch(self.table_sets[req.geometry], np.zeros(n, np.int32), np.full(n, net.kT), None, None,
                              np.tile(net.occupation.astype(np.uint8), (n, 1)), np.full(n, req.hops),
                              seed=req.seed, lanes=self.lanes, dev=self.dev, E_constant_dev=ec,
                              el_energy_dev=ve, pair_mode=self.pair_mode)
        req.bytes = need
        self.mem_used += need
        self.active.append(req)

    def _launch_ready(self):
        # least remaining work first
        for req in sorted(self.active, key=lambda r: r.hops - r.launched_hops):
            if req.launched_hops >= req.hops:
                continue
            if req.inflight is not None and not req.inflight.query():
                continue
            seg = min(self.quantum, req.hops - req.launched_hops)
            seg_launch = ((seg + _REANCHOR - 1) // _REANCHOR) * _REANCHOR
            with torch.cuda.stream(req.stream):
                req.batch.launch(seg_launch, stream=req.stream)
                ev = torch.cuda.Event()
                ev.record(req.stream)
            req.inflight = ev
            req.launched_hops += seg
            req.started = True

    def _collect(self):
        still = []
        for req in self.active:
            if req.launched_hops >= req.hops and req.inflight is not None and req.inflight.query():
                r = req.batch.results()
                cur = np.array([e / t if t > 0 else np.full(len(e), np.nan)
                                for e, t in zip(r["electrode_occupation"], r["time"])])
                req.done_at = time.perf_counter()
                self.hops_done += int(np.sum(r["hops_done"]))
                out = dict(currents=cur, time=r["time"], electrode_occupation=np.array(r["electrode_occupation"]),
                           status=r["status"], latency=req.done_at - req.arrival)
                self.mem_used -= req.bytes
                req.batch = None
                self.finished.append(req)
                req.future.set_result(out)
            else:
                still.append(req)
        self.active = still

    def _loop(self):
        torch.cuda.set_device(self.dev)
        while True:
            with self.cv:
                while not self._stop and not self.queue and not self.active:
                    self.cv.wait(0.05)
                if self._stop and not self.queue and not self.active:
                    return
                self._admit()
            self._launch_ready()
            self._collect()
            time.sleep(0)

    def run_sync(self):
        """Run everything queued to completion in the calling thread."""
        torch.cuda.set_device(self.dev)
        while True:
            with self.lock:
                self._admit()
                if not self.queue and not self.active:
                    return
            self._launch_ready()
            self._collect()


def latency_summary(requests):
    """p50 / p99 latency (ms) overall and per hop budget."""
    out = {}
    lat = np.array([r.done_at - r.arrival for r in requests if r.done_at is not None])
    if lat.size:
        out["all"] = dict(n=int(lat.size), p50_ms=float(np.percentile(lat, 50) * 1e3),
                          p99_ms=float(np.percentile(lat, 99) * 1e3))
    for h in sorted({r.hops for r in requests}):
        l = np.array([r.done_at - r.arrival for r in requests if r.hops == h and r.done_at is not None])
        if l.size:
            out[f"hops_{h}"] = dict(n=int(l.size), p50_ms=float(np.percentile(l, 50) * 1e3),
                                    p99_ms=float(np.percentile(l, 99) * 1e3))
    return out
