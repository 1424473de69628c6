"""Python face of the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke`` and bench.py's CPU-baseline legs use
this module; it checks the CUDA kernels and is never the thing measured as
the product.  It wraps the C restatement in kmc_oracle.c (built by
oracle/build.py) and adds a small pure-Python restatement of the numba hop
loop (kmc_dopant_networks.py:33-135) for cross-checking the C one on tiny
cases.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build as _build  # noqa: E402

_LIB = None
_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(_build.build())
        L.oracle_numba_replay.restype = C.c_int
        L.oracle_numba_replay.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                          C.c_double, _u8p, _dp, _dp, _dp, _dp, _i64p, C.c_int64,
                                          C.c_int, _dp, _dp, _dp, _dp, _i32p, _dp, _dp, _dp, _dp]
        L.oracle_clear_stream.restype = C.c_int
        L.oracle_clear_stream.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                          C.c_double, _u8p, _dp, _dp, _dp, _dp, C.c_int64, C.c_uint64,
                                          C.c_double, _dp, _i64p]
        L.oracle_go_simulate.restype = C.c_double
        L.oracle_go_simulate.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                         C.c_double, _u8p, _dp, _dp, _dp, _dp, _dp, C.c_int64,
                                         C.c_int, _dp, _dp, C.c_uint64, _i64p]
        L.oracle_go_chains.restype = C.c_int
        L.oracle_go_chains.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.c_double, _u8p, _dp, _dp, _dp, _dp, C.c_int64, C.c_int64,
                                       C.c_int64, C.c_uint64, _dp, _dp, _i64p]
        L.oracle_prob_simulate.restype = C.c_double
        L.oracle_prob_simulate.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                           C.c_double, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int, C.c_int,
                                           _dp, _dp]
        _LIB = L
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def numba_replay(N, P, nu, kT, I_0, R, occupation, distances, E_constant, site_energies,
                 transitions_constant, uniforms, hops=None, record=True, electrode_occupation=None):
    """FP64 restatement of _simulate_discrete_record with a replay stream.

    Returns dict(time, occupation, electrode_occupation, traffic,
    occupations_in_time, hop_log (hops, 2), hop_times, margins, hop_totals
    (the total rate of each hop's state), hop_rates (the chosen pair's
    rate))."""
    S = N + P
    hops = len(uniforms) // 2 if hops is None else int(hops)
    occ = np.ascontiguousarray(occupation, dtype=np.uint8).copy()
    eo = (np.zeros(P, np.int64) if electrode_occupation is None
          else np.ascontiguousarray(electrode_occupation, dtype=np.int64).copy())
    d = np.ascontiguousarray(distances, dtype=np.float64)
    tc = np.ascontiguousarray(transitions_constant, dtype=np.float64)
    ec = np.ascontiguousarray(E_constant, dtype=np.float64)
    se = np.ascontiguousarray(site_energies, dtype=np.float64)
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    traffic = np.zeros((S, S))
    oit = np.zeros(max(N, 1))
    log = np.zeros((hops, 2), np.int32)
    ht = np.zeros(hops)
    mg = np.zeros(hops)
    tot = np.zeros(hops)
    rch = np.zeros(hops)
    t = C.c_double(0)
    rc = lib().oracle_numba_replay(N, P, nu, kT, I_0, R, _p(occ, _u8p), _p(d, _dp), _p(ec, _dp),
                                   _p(se, _dp), _p(tc, _dp), _p(eo, _i64p), hops, int(record),
                                   _p(u, _dp), C.byref(t), _p(traffic, _dp), _p(oit, _dp),
                                   _p(log, _i32p), _p(ht, _dp), _p(mg, _dp), _p(tot, _dp), _p(rch, _dp))
    if rc != 0:
        raise RuntimeError(f"oracle_numba_replay failed: {rc}")
    return dict(time=t.value, occupation=occ, electrode_occupation=eo, traffic=traffic,
                occupations_in_time=oit[:N], hop_log=log, hop_times=ht, margins=mg,
                hop_totals=tot, hop_rates=rch)


def clear_stream(N, P, nu, kT, I_0, R, occupation, distances, E_constant, site_energies,
                 transitions_constant, hops, seed, min_margin=1e-4):
    """A replay stream (2*hops uniforms) on which every hop of the numba
    loop started from ``occupation`` selects its pair with the event uniform
    at least ``min_margin`` of the total rate away from that pair's
    cumulative boundaries (close uniforms are redrawn).  Returns (uniforms,
    number of redraws)."""
    u = np.zeros(2 * int(hops))
    nre = C.c_int64(0)
    rc = lib().oracle_clear_stream(
        N, P, nu, kT, I_0, R, _p(np.ascontiguousarray(occupation, dtype=np.uint8), _u8p),
        _p(np.ascontiguousarray(distances, np.float64), _dp), _p(np.ascontiguousarray(E_constant, np.float64), _dp),
        _p(np.ascontiguousarray(site_energies, np.float64), _dp),
        _p(np.ascontiguousarray(transitions_constant, np.float64), _dp), int(hops),
        C.c_uint64(int(seed) & (2**64 - 1)), float(min_margin), _p(u, _dp), C.byref(nre))
    if rc != 0:
        raise RuntimeError(f"oracle_clear_stream failed: {rc}")
    return u, nre.value


def go_simulate(N, P, nu, kT, I_0, R, occupation, distances, E_constant, site_energies,
                transitions_constant, hops, seed, record=False):
    """FP32 restatement of Go simulate() (no memo) for one chain."""
    S = N + P
    occ = np.ascontiguousarray(occupation, dtype=np.uint8).copy()
    eo = np.zeros(P)
    traffic = np.zeros((S, S))
    avg = np.zeros(max(N, 1))
    na = C.c_int64(0)
    t = lib().oracle_go_simulate(
        N, P, nu, kT, I_0, R, _p(occ, _u8p), _p(np.ascontiguousarray(distances, np.float64), _dp),
        _p(np.ascontiguousarray(E_constant, np.float64), _dp),
        _p(np.ascontiguousarray(site_energies, np.float64), _dp),
        _p(np.ascontiguousarray(transitions_constant, np.float64), _dp), _p(eo, _dp), int(hops),
        int(record), _p(traffic, _dp), _p(avg, _dp), C.c_uint64(seed & (2**64 - 1)), C.byref(na))
    return dict(time=t, occupation=occ, electrode_occupation=eo, traffic=traffic,
                average_occupation=avg[:N], n_allowed=na.value)


def prob_simulate(N, P, nu, kT, I_0, R, occupation, distances, E_constant, site_energies,
                  transitions_constant, hops, record=False):
    """FP64 restatement of Go probSimulate (mean-field relaxation) for one
    network; ``occupation`` (N probabilities) is the starting point (the Go
    wrapper passes 0.5 everywhere).  ``site_energies`` has S entries, the
    electrode ones being the voltages."""
    S = N + P
    occ = np.array(occupation, dtype=np.float64, copy=True)
    se = np.array(site_energies, dtype=np.float64, copy=True)
    eo = np.zeros(max(P, 1))
    traffic = np.zeros((S, S))
    avg = np.zeros(max(N, 1))
    t = lib().oracle_prob_simulate(
        N, P, nu, kT, I_0, R, _p(occ, _dp), _p(np.ascontiguousarray(distances, np.float64), _dp),
        _p(np.ascontiguousarray(E_constant, np.float64), _dp),
        _p(np.ascontiguousarray(transitions_constant, np.float64), _dp), _p(eo, _dp), _p(se, _dp),
        int(hops), int(record), _p(traffic, _dp), _p(avg, _dp))
    return dict(time=t, occupation=occ, electrode_occupation=eo[:P], site_energies=se,
                traffic=traffic, average_occupation=avg[:N])


def go_chains(N, P, nu, kT, I_0, R, occupations, distances, E_constant_rows, site_energy_rows,
              transitions_constant, hops, seed, threads=None):
    """Many chains on one geometry, split across host threads (ctypes drops
    the GIL during each call).  Returns (times[C], eo[C, P], n_allowed[C])."""
    occ = np.ascontiguousarray(occupations, dtype=np.uint8)
    n = occ.shape[0]
    d = np.ascontiguousarray(distances, np.float64)
    tc = np.ascontiguousarray(transitions_constant, np.float64)
    ec = np.ascontiguousarray(E_constant_rows, np.float64)
    se = np.ascontiguousarray(site_energy_rows, np.float64)
    times = np.zeros(n)
    eo = np.zeros((n, P))
    na = np.zeros(n, np.int64)
    threads = threads or os.cpu_count() or 1
    threads = max(1, min(threads, n))
    bounds = np.linspace(0, n, threads + 1).astype(np.int64)
    L = lib()

    def work(k):
        a, b = int(bounds[k]), int(bounds[k + 1])
        if b > a:
            rc = L.oracle_go_chains(N, P, nu, kT, I_0, R, _p(occ, _u8p), _p(d, _dp), _p(ec, _dp),
                                    _p(se, _dp), _p(tc, _dp), int(hops), a, b - a,
                                    C.c_uint64(seed & (2**64 - 1)), _p(times, _dp), _p(eo, _dp),
                                    _p(na, _i64p))
            if rc != 0:
                raise RuntimeError("oracle_go_chains failed")
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, range(threads)))
    return times, eo, na


def numba_replay_py(N, P, nu, kT, I_0, R, occupation, distances, E_constant, site_energies,
                    transitions_constant, uniforms):
    """Pure-Python restatement of the same loop for tiny cases (hop log only)."""
    S = N + P
    occ = [bool(x) for x in occupation]
    se = list(map(float, site_energies))
    log, t = [], 0.0
    for hop in range(len(uniforms) // 2):
        for i in range(N):
            acc = 0
            for j in range(N):
                if j != i:
                    acc += (1 - occ[j]) / distances[i][j]
            se[i] = float(E_constant[i])
            se[i] += -I_0 * R * acc
        cum, run = [], 0.0
        for i in range(S):
            for j in range(S):
                if (i >= N and j >= N) or (i >= N and occ[j]) or (j >= N and i < N and not occ[i]) \
                        or (i < N and j < N and (i == j or not occ[i] or occ[j])):
                    r = 0.0
                else:
                    dE = se[j] - se[i] - (I_0 * R / distances[i][j] if (i < N and j < N) else 0.0)
                    r = nu * np.exp(-dE / kT) if dE > 0 else nu
                r = transitions_constant[i][j] * r
                run = r if (i == 0 and j == 0) else r + run
                cum.append(run)
        total = cum[-1]
        t += -np.log(1 - uniforms[2 * hop]) * (1 / total)
        u = uniforms[2 * hop + 1]
        ev = next(k for k in range(S * S) if cum[k] / total >= u)
        fr, to = divmod(ev, S)
        if fr < N:
            occ[fr] = False
        if to < N:
            occ[to] = True
        log.append((fr, to))
    return np.array(log, np.int32), t


def prob_simulate_py(N, P, nu, kT, I_0, R, occupation, distances, E_constant, site_energies,
                     transitions_constant, hops, record=False):
    """Plain-Python restatement of Go probSimulate (probabilitySimulation.go:
    53-157), loop for loop; small cases only.  Cross-checks the C oracle."""
    import math
    S = N + P
    occ = [float(x) for x in occupation]
    se = [float(x) for x in site_energies]
    d = np.asarray(distances, np.float64).reshape(S, S).tolist()
    tc = np.asarray(transitions_constant, np.float64).reshape(S, S).tolist()
    Ec = [float(x) for x in E_constant]
    eo = [0.0] * P
    traffic = [0.0] * (S * S)
    avg = [0.0] * N
    t = [[0.0] * S for _ in range(S)]
    time = 0.0
    for _ in range(int(hops)):
        diff = [0.0] * N
        for i in range(N):
            acc = 0.0
            for j in range(N):
                if j != i:
                    acc += (1 - occ[j]) / d[i][j]
            se[i] = Ec[i] - I_0 * R * acc
        tot = 0.0
        for i in range(S):
            for j in range(S):
                if i >= N and j >= N:
                    base = 0.0
                elif i >= N:
                    base = 1 - occ[j]
                elif j >= N:
                    base = occ[i]
                else:
                    base = (1 - occ[j]) * occ[i]
                if i < N and j < N:
                    dE = se[j] - se[i] - I_0 * R / d[i][j] if d[i][j] != 0 else -math.inf
                else:
                    dE = se[j] - se[i]
                r = base * nu * math.exp(-dE / kT) if dE > 0 else base * nu
                r *= tc[i][j]
                t[i][j] = r
                tot += r
                if i < N:
                    diff[i] -= r
                if j < N:
                    diff[j] += r
        mc = 1.0
        for i in range(N):
            nv = occ[i] + diff[i] / tot
            if nv < 0:
                req = occ[i] / -(diff[i] / tot)
                if req < mc:
                    mc = req
            if nv > 1:
                req = (1 - occ[i]) / (diff[i] / tot)
                if req < mc:
                    mc = req
        step = 0.98 * mc / tot
        time += step
        if record:
            for i in range(N):
                avg[i] += occ[i] * step
        for i in range(S):
            for j in range(S):
                if i >= N and j >= N:
                    break
                rate = t[i][j] * mc / tot
                if i < N:
                    occ[i] -= rate
                else:
                    eo[i - N] -= rate
                if j < N:
                    occ[j] += rate
                else:
                    eo[j - N] += rate
                if record:
                    traffic[i * S + j] += rate
                    traffic[j * S + i] -= rate
        for i in range(N):
            occ[i] = min(max(occ[i], 0.0), 1.0) if not (occ[i] != occ[i]) else occ[i]
    return dict(time=time, occupation=np.array(occ), electrode_occupation=np.array(eo),
                site_energies=np.array(se), traffic=np.array(traffic).reshape(S, S),
                average_occupation=np.array(avg))
