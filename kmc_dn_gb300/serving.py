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
* admits waiting requests, least work first (chains x hops x pairs per
  hop), while their chain state fits the device memory budget; long
  requests (more than ``short_hops`` hops) may occupy at most
  ``long_thread_share`` of the device's resident-thread slots (chains x
  threads per chain), so a short request is admitted on arrival and finds
  room on the SMs instead of queueing behind minutes of long work;
  admitted state stays resident until the request is done;
* runs every admitted request in quanta of hops on a CUDA stream of its own
  (pooled and reused), so requests that arrive while others run are started
  at once, their launches overlap on the device, and reading a finished
  request's results waits for nothing else; the request with the least
  remaining work is launched first, short requests use high-priority
  streams and wider thread groups, and long requests run in shorter quanta
  so that the blocks a short request waits for free up within a few
  milliseconds; while a short request waits or runs, long requests get no
  new quantum at all (strict priority, with a starvation guard), so the
  short one has the device to itself once the long quanta in flight end;
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
from .engine import Batch, CancelWord, TableSet, TableSpec, _REANCHOR, superpose

__all__ = ["Request", "Server", "latency_summary"]

# Resident threads per SM of the engine's kernels at their register budgets
# (block groups: 2 blocks of 256 threads at <= 128 registers).
_ENGINE_THREADS_PER_SM = 512


@dataclass(eq=False)          # identity: queue removal must not compare voltage arrays
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
    cancel_word: Optional[object] = None   # engine.CancelWord while the request is active
    cancelled: bool = False
    paused_since: Optional[float] = None   # a long request held back for short ones since


def _request_bytes(n_chains, N, P):
    # per chain: energies (4N) + occupation (N) + electrode energies (4P) and
    # counters (8P) + time/hops/stream/status/pairs (48) + work slot (4)
    return n_chains * (5 * N + 12 * P + 52)


class Server:
    """Serve hop-loop requests on one GPU with continuous batching.

    networks:       list of workloads.Network (the resident geometries)
    quantum:        hops per launch of a short request (a multiple of 1024)
    quantum_long:   hops per launch of a long request (default 1024)
    short_lanes_factor: short requests run with this many times the default
                    threads per chain (lower latency, lower throughput)
    short_thread_share: a short request's chains x threads per chain stay
                    within this share of the engine's resident threads (512
                    per SM at its register budgets), narrowing the groups of
                    a large request, so that the next short request finds
                    free SMs instead of waiting for a launch that fills them
    short_big_quantum: hops per launch of a short request that holds at
                    least half of that cap (a multiple of 1024; default
                    2048): its blocks free up between quanta, where the next
                    short request (less work, launched first) takes them
    short_hops:     requests with at most this many hops are short
    long_thread_share: fraction of the device's resident-thread slots that
                    long requests may hold (default 0.75)
    max_long_pause: seconds a long request may be held back while short
                    requests run (strict priority) before it gets a quantum
    max_active_chains:      resident chains in all
    mem_budget:     bytes of chain state admitted at once (default: a
                    quarter of the free device memory at start)
    pair_mode:      "positions" (tables must be those of the positions) or
                    "table"
    """

    def __init__(self, networks, *, quantum=4096, mem_budget=None,
                 pair_mode="positions", lanes=None, dev=None, short_hops=20000,
                 max_active_chains=16384, long_thread_share=0.75, quantum_long=_REANCHOR,
                 short_lanes_factor=4, max_long_pause=1.0, short_thread_share=0.5,
                 short_big_quantum=2048):
        if quantum % _REANCHOR or quantum_long % _REANCHOR or quantum_long <= 0 or \
                short_big_quantum % _REANCHOR or short_big_quantum <= 0:
            raise ValueError("quanta must be positive multiples of the re-anchor period (1024)")
        d = torch.device(dev if dev is not None else "cuda")
        self.dev = torch.device("cuda", d.index if d.index is not None else torch.cuda.current_device())
        self.networks = list(networks)
        self.quantum = int(quantum)
        self.quantum_long = int(quantum_long)
        self.short_big_quantum = int(short_big_quantum)
        self.pair_mode = pair_mode
        self.lanes = lanes
        self.short_lanes_factor = int(short_lanes_factor)
        self.short_hops = int(short_hops)
        self.max_long_pause = float(max_long_pause)
        free, _total = torch.cuda.mem_get_info(self.dev)
        self.mem_budget = int(mem_budget if mem_budget is not None else free // 4)
        self.mem_used = 0
        self.max_active_chains = int(max_active_chains)
        props = torch.cuda.get_device_properties(self.dev)
        self.long_thread_budget = int(long_thread_share * props.multi_processor_count
                                      * props.max_threads_per_multi_processor)
        self.short_thread_cap = int(short_thread_share * props.multi_processor_count * _ENGINE_THREADS_PER_SM)
        self.active_chains = 0
        self.active_long_chains = 0
        self.active_long_threads = 0
        lo, hi = torch.cuda.Stream.priority_range()
        # every active request owns a stream (no request waits behind another's
        # launches); finished requests return theirs to a pool per priority
        self._prio = {True: hi, False: lo}
        self._free_streams = {True: [], False: []}
        self.n_streams_created = 0
        self.specs = [TableSpec.from_network(n) for n in self.networks]
        # one resident table set per geometry (a request names one geometry)
        self.table_sets = [TableSet([sp], pair_mode=pair_mode, dev=self.dev) for sp in self.specs]
        self.queue = deque()
        self.active = []
        self.finished = []
        self.lock = threading.Lock()
        self.cv = threading.Condition(self.lock)
        # one thread at a time admits, launches and collects (the server
        # thread, or the caller of run_sync / wait_idle when none runs)
        self._drive = threading.Lock()
        self._thread = None
        self._stop = False
        self._error = None
        self.hops_done = 0
        self.launches = 0         # kernels launched (site energies + engine)

    # ---------------------------------------------------------------- API
    def submit(self, geometry, voltages, hops, seed):
        V = np.asarray(voltages, np.float64)
        if V.ndim != 2 or V.shape[1] != self.networks[geometry].P:
            raise ValueError("voltages must be (n_chains, P) for the geometry")
        if not np.isfinite(V).all():
            # the hop loop, like the reference's, treats a NaN energy
            # difference as downhill and would run on silently: refuse here
            raise ValueError("voltages must be finite")
        req = Request(int(geometry), V, int(hops), int(seed), arrival=time.perf_counter())
        with self.cv:
            self.queue.append(req)
            self.cv.notify()
        return req

    def cancel(self, req):
        """Cancel a request: a waiting one is dropped, an active one stops
        its chains at their next 1024-hop check (a host-mapped cancel word
        its kernels poll) and is finished with what it has; either way its
        future gets a result with ``cancelled`` True and the chains'
        status (KMC_ERR_CANCELLED for the stopped ones)."""
        with self.lock:
            if req in self.queue:
                self.queue.remove(req)
                req.cancelled = True
                req.done_at = time.perf_counter()
                req.future.set_result(dict(cancelled=True, status=np.full(req.voltages.shape[0],
                                                                          _native.KMC_ERR_CANCELLED, np.int32)))
                return True
            if any(r is req for r in self.active):
                req.cancelled = True
                if req.cancel_word is not None:
                    req.cancel_word.set()
                return True
        return False

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
        self._raise_error()

    def wait_idle(self, timeout=None):
        """Until every submitted request is finished (True), or `timeout`
        seconds passed (False).  With the server thread running this only
        waits; otherwise it drives the requests itself."""
        t0 = time.perf_counter()
        while True:
            self._raise_error()
            with self.lock:
                if not self.queue and not self.active:
                    return True
            if timeout is not None and time.perf_counter() - t0 > timeout:
                return False
            if self._thread is not None and self._thread.is_alive():
                time.sleep(0.0005)
            else:
                self._step()

    def run_sync(self):
        """Run everything queued to completion in the calling thread."""
        torch.cuda.set_device(self.dev)
        while True:
            with self.lock:
                if not self.queue and not self.active:
                    return
            self._step()

    # ----------------------------------------------------------- internals
    def _work(self, req):
        net = self.networks[req.geometry]
        h = 0.9 * net.N           # typical hole count: pairs per hop ~ A(h)
        pairs = h * (net.N - h) + h * net.P + net.P * (net.N - h)
        return req.voltages.shape[0] * req.hops * pairs

    def _lanes(self, req):
        """Threads per chain: the throughput default, or for a short request
        a wider group (its latency is hops x per-hop time, and a wider group
        cuts the per-hop time), narrowed while the request's chains would
        hold more than short_thread_cap threads: a request that fills the
        SMs holds every block slot until its launch ends, and a wider group
        past that point only adds waves."""
        if self.lanes is not None:
            return self.lanes
        if req.hops > self.short_hops or self.short_lanes_factor <= 1:
            return None
        from .engine import default_lanes
        net = self.networks[req.geometry]
        G = min(512, default_lanes(net.N + net.P) * self.short_lanes_factor)
        n = req.voltages.shape[0]
        while G > 4 and n * G > self.short_thread_cap:
            G //= 2
        return G

    def _quantum(self, req):
        """Hops per launch: long requests short quanta; short ones one launch,
        or short_big_quantum when they hold half the short-thread cap."""
        if req.hops > self.short_hops:
            return self.quantum_long
        if 2 * self._threads(req) >= self.short_thread_cap:
            return min(self.quantum, self.short_big_quantum)
        return self.quantum

    def _threads(self, req):
        """Resident threads the request's chains occupy."""
        from .engine import default_lanes
        net = self.networks[req.geometry]
        G = self._lanes(req) or default_lanes(net.N + net.P)
        return req.voltages.shape[0] * G

    def _admit(self):
        if not self.queue:
            return
        waiting = sorted(self.queue, key=self._work)
        for req in waiting:
            net = self.networks[req.geometry]
            n = req.voltages.shape[0]
            need = _request_bytes(n, net.N, net.P)
            long_ = req.hops > self.short_hops
            if self.active:
                if self.mem_used + need > self.mem_budget or self.active_chains + n > self.max_active_chains:
                    break
                if long_ and self.active_long_threads > 0 and \
                        self.active_long_threads + self._threads(req) > self.long_thread_budget:
                    continue        # a shorter request further down may still fit
            self.queue.remove(req)
            self._prepare(req, need)

    def _prepare(self, req, need):
        net = self.networks[req.geometry]
        n = req.voltages.shape[0]
        short = req.hops <= self.short_hops
        pool = self._free_streams[short]
        if pool:
            req.stream = pool.pop()
        else:
            req.stream = torch.cuda.Stream(device=self.dev, priority=self._prio[short])
            self.n_streams_created += 1
        with torch.cuda.stream(req.stream):
            ec, ve = superpose(net.basis, net.comp, req.voltages, net.mu, dev=self.dev, stream=req.stream)
            req.batch = Batch(self.table_sets[req.geometry], np.zeros(n, np.int32), np.full(n, net.kT), None, None,
                              np.tile(net.occupation.astype(np.uint8), (n, 1)), np.full(n, req.hops),
                              seed=req.seed, lanes=self._lanes(req), dev=self.dev, E_constant_dev=ec,
                              el_energy_dev=ve, pair_mode=self.pair_mode)
        req.cancel_word = CancelWord()
        req.batch.cancel = req.cancel_word
        self.launches += 1
        req.bytes = need
        self.mem_used += need
        self.active_chains += n
        if req.hops > self.short_hops:
            self.active_long_chains += n
            self.active_long_threads += self._threads(req)
        self.active.append(req)

    def _short_busy(self):
        """A short request is waiting, or active with work left to run."""
        if any(r.hops <= self.short_hops for r in self.queue):
            return True
        return any(r.hops <= self.short_hops and r.launched_hops < r.hops and not r.cancelled
                   for r in self.active)

    def _may_launch(self, req, short_busy, now):
        """Strict priority for short requests: while one waits or runs, long
        requests get no new quantum (the quanta in flight end within one
        quantum, so a short request soon has the device to itself).  A long
        request paused for more than max_long_pause seconds gets one quantum
        all the same, so that a steady stream of short requests cannot
        starve it."""
        if req.hops <= self.short_hops or not short_busy:
            req.paused_since = None
            return True
        if req.paused_since is None:
            req.paused_since = now
        if now - req.paused_since > self.max_long_pause:
            req.paused_since = None
            return True
        return False

    def _launch_ready(self):
        short_busy = self._short_busy()
        now = time.perf_counter()
        # least remaining work first
        for req in sorted(self.active, key=lambda r: r.hops - r.launched_hops):
            if req.launched_hops >= req.hops or req.cancelled:
                continue
            if req.inflight is not None and not req.inflight.query():
                continue
            if not self._may_launch(req, short_busy, now):
                continue
            q = self._quantum(req)
            seg = min(q, req.hops - req.launched_hops)
            seg_launch = ((seg + _REANCHOR - 1) // _REANCHOR) * _REANCHOR
            with torch.cuda.stream(req.stream):
                # an NVTX range per launch: profilers show which request ran when
                torch.cuda.nvtx.range_push(f"kmc g{req.geometry} c{req.voltages.shape[0]} "
                                           f"hops {req.launched_hops}+{seg}")
                req.batch.launch(seg_launch, stream=req.stream)
                torch.cuda.nvtx.range_pop()
                self.launches += len(req.batch._bins)
                ev = torch.cuda.Event()
                ev.record(req.stream)
            req.inflight = ev
            req.launched_hops += seg
            req.started = True

    def _collect(self):
        still = []
        for req in self.active:
            finished = req.launched_hops >= req.hops or req.cancelled
            if finished and (req.inflight is None or req.inflight.query()):
                r = req.batch.results(stream=req.stream)
                cur = np.array([e / t if t > 0 else np.full(len(e), np.nan)
                                for e, t in zip(r["electrode_occupation"], r["time"])])
                req.done_at = time.perf_counter()
                self.hops_done += int(np.sum(r["hops_done"]))
                status = r["status"].copy()
                if req.cancelled:
                    # a cancel that lands between two quanta stops the chains
                    # before the next launch, which then never polls the
                    # cancel word: they are cancelled all the same
                    status[(status == _native.KMC_OK) & (r["hops_done"] < req.hops)] = _native.KMC_ERR_CANCELLED
                out = dict(currents=cur, time=r["time"], electrode_occupation=np.array(r["electrode_occupation"]),
                           status=status, latency=req.done_at - req.arrival, cancelled=req.cancelled,
                           hops_done=r["hops_done"])
                self.mem_used -= req.bytes
                self.active_chains -= req.voltages.shape[0]
                if req.hops > self.short_hops:
                    self.active_long_chains -= req.voltages.shape[0]
                    self.active_long_threads -= self._threads(req)
                req.batch = None
                if req.cancel_word is not None:
                    req.cancel_word.close()
                    req.cancel_word = None
                self._free_streams[req.hops <= self.short_hops].append(req.stream)
                self.finished.append(req)
                req.future.set_result(out)
            else:
                still.append(req)
        self.active = still

    def _step(self):
        with self._drive:
            with self.lock:
                self._admit()
            self._launch_ready()
            self._collect()

    def _raise_error(self):
        if self._error is not None:
            raise RuntimeError("serving loop failed") from self._error

    def _loop(self):
        try:
            torch.cuda.set_device(self.dev)
            while True:
                with self.cv:
                    while not self._stop and not self.queue and not self.active:
                        self.cv.wait(0.05)
                    if self._stop and not self.queue and not self.active:
                        return
                self._step()
                time.sleep(0)
        except BaseException as e:      # fail the waiting callers instead of leaving them waiting
            self._error = e
            with self.lock:
                pending = list(self.queue) + list(self.active)
                self.queue.clear()
                self.active = []
            for req in pending:
                if not req.future.done():
                    req.future.set_exception(e)



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
