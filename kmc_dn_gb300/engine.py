"""Host side of the hop-loop kernels: device buffers, launches, results.

Device memory and streams come from PyTorch (tensors are only buffers); the
computation is the CUDA kernels behind the C ABI (``_native``).  Nothing here
computes hops on the CPU.

* ``simulate_f64``   -- one chain through the plain FP64 kernel (numba
                        semantics; optional replay stream and hop log).
* ``Batch``          -- many chains through the batched FP32 engine: pair
                        tables shared by chains of one geometry, per-chain
                        state resident on the device, chains binned by size
                        into launches with their own lanes-per-chain.
* ``simulate_cuda``  -- keyword-compatible replacement of the reference's
                        ``_simulate_discrete_record`` / ``callGoSimulation``
                        (kmc_dopant_networks.py:33-135, goSimulation/
                        pythonBind.py:49-92) for ``makeSimulation``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np
import torch

from . import _native
from ._native import check, lib

__all__ = ["simulate_f64", "TableSpec", "TableSet", "Batch", "simulate_cuda", "simulate_go", "superpose",
           "default_lanes", "make_work_lists", "device", "prune", "CancelWord", "simulate_f64_many",
           "balanced_warps_per_block", "widen_small_launch"]


_PRELOADED = set()


def device(dev=None):
    """The CUDA device to run on; on first use of a device every kernel of
    the library is loaded there (kmc_preload_kernels), so that no launch
    waits on a lazy code load behind the kernels already running."""
    if not torch.cuda.is_available():
        raise RuntimeError("kmc_dn_gb300 needs a CUDA device: the hop loop runs only as CUDA kernels")
    d = torch.device(dev if dev is not None else "cuda")
    idx = d.index if d.index is not None else torch.cuda.current_device()
    if idx not in _PRELOADED:
        with torch.cuda.device(idx):
            check(lib().kmc_preload_kernels())
        _PRELOADED.add(idx)
    return d


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _dev(a, dtype, dev):
    # contiguous and writable (a broadcast view is read-only; torch warns on those)
    return torch.as_tensor(np.require(a, requirements=("C", "W")), dtype=dtype).to(dev)


# ---------------------------------------------------------------------------
# plain FP64 single chain
# ---------------------------------------------------------------------------

def simulate_f64(N, P, nu, kT, I_0, R, occupation, distances, E_constant, site_energies,
                 transitions_constant, hops, *, electrode_occupation=None, record=False,
                 uniforms=None, seed=0, hop_log=False, dev=None, stream=None, flux=False):
    """Run one chain on the plain FP64 kernel.

    Returns dict(time, occupation, electrode_occupation, traffic,
    occupations_in_time, hop_log, status[, flux_time]).  ``uniforms``
    (2*hops values in (0,1)) switches on replay mode; ``flux`` adds the time
    integral of each electrode's expected net inflow."""
    d = device(dev)
    S = N + P
    hops = int(hops)
    f64 = torch.float64
    occ = _dev(np.asarray(occupation, dtype=np.uint8).reshape(N), torch.uint8, d)
    dist = _dev(np.asarray(distances, np.float64).reshape(S, S), f64, d)
    tc = _dev(np.asarray(transitions_constant, np.float64).reshape(S, S), f64, d)
    ec = _dev(np.asarray(E_constant, np.float64).reshape(N), f64, d)
    se = _dev(np.asarray(site_energies, np.float64).reshape(S), f64, d)
    eo0 = np.zeros(P, np.int64) if electrode_occupation is None else np.asarray(electrode_occupation, np.int64)
    eo = _dev(eo0.reshape(P), torch.int64, d)
    traffic = torch.zeros((S, S), dtype=f64, device=d) if record else None
    oit = torch.zeros(max(N, 1), dtype=f64, device=d) if record else None
    u = None
    if uniforms is not None:
        u = _dev(np.asarray(uniforms, np.float64), f64, d)
        if u.numel() < 2 * hops:
            raise ValueError("replay stream shorter than 2*hops")
    log = torch.zeros(2 * max(hops, 1), dtype=torch.int32, device=d) if hop_log else None
    t_out = torch.zeros(1, dtype=f64, device=d)
    st_out = torch.zeros(1, dtype=torch.int32, device=d)
    L = lib()
    wsb = L.kmc_simulate_f64_workspace_size(S)
    ws = torch.empty(max(wsb, 8), dtype=torch.uint8, device=d)
    fx = torch.zeros(max(P, 1), dtype=f64, device=d) if flux else None
    args = (N, P, float(nu), float(kT), float(I_0), float(R), _ptr(occ), _ptr(dist),
            _ptr(ec), _ptr(se), _ptr(tc), _ptr(eo), hops, int(bool(record)),
            _ptr(traffic), _ptr(oit), _ptr(u), int(seed) & (2**64 - 1), _ptr(log),
            _ptr(t_out), _ptr(st_out), _ptr(ws), wsb, _stream_handle(stream))
    if flux:
        check(L.kmc_simulate_f64_flux(*args, _ptr(fx)))
    else:
        check(L.kmc_simulate_f64(*args))
    torch.cuda.synchronize(d)
    out = dict(time=float(t_out.item()), occupation=occ.cpu().numpy().astype(bool),
               electrode_occupation=eo.cpu().numpy(), status=int(st_out.item()))
    out["traffic"] = traffic.cpu().numpy() if record else np.zeros((S, S))
    out["occupations_in_time"] = oit.cpu().numpy()[:N] if record else np.zeros(N)
    if hop_log:
        out["hop_log"] = log.cpu().numpy()[: 2 * hops].reshape(hops, 2)
    if flux:
        out["flux_time"] = fx.cpu().numpy()[:P]
    return out


class CancelWord:
    """A flag the host sets while kernels run (pinned, mapped host memory,
    kmc_cancel_word_create).  Give it to ``Batch.cancel``: after ``set()``
    every chain of that batch's running and later launches stops at its next
    1024-hop check with KMC_ERR_CANCELLED, its state consistent (``clear()``
    and a further launch resume it as if uninterrupted)."""

    def __init__(self):
        h, d = C.c_void_p(), C.c_void_p()
        check(lib().kmc_cancel_word_create(C.byref(h), C.byref(d)))
        self._host = C.cast(h, C.POINTER(C.c_int32))
        self._h = h
        self.device = d.value

    def set(self):
        self._host[0] = 1

    def clear(self):
        self._host[0] = 0

    def is_set(self):
        return bool(self._host[0])

    def close(self):
        if self._h is not None:
            lib().kmc_cancel_word_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def simulate_f64_many(chains, hops, seeds, *, dev=None, record=False, flux=False, n_streams=None):
    """Run independent FP64 chains of the plain FP64 kernel in one launch
    (kmc_simulate_f64_batch: one block per chain), for FP64 reference
    statistics.

    ``chains``: list of dicts with N, P, nu, kT, I_0, R, occupation,
    distances, E_constant, site_energies, transitions_constant (chains
    whose distances / transitions_constant are the same arrays share one
    device copy).  ``hops``: one budget or one per chain.  Returns
    (time[C], electrode_occupation[C][P], status[C]) and, with ``record``,
    a fourth list: occupations_in_time[C][N] (numba convention); with
    ``flux`` a last list: the time integral of each electrode's expected net
    inflow.  (``n_streams`` is accepted for compatibility and unused.)"""
    d = device(dev)
    f64, i64 = torch.float64, torch.int64
    n = len(chains)
    if n == 0:
        return (np.zeros(0), [], np.zeros(0, np.int32)) + (([],) if record else ()) + (([],) if flux else ())
    Ns = np.array([int(ch["N"]) for ch in chains], np.int32)
    Ps = np.array([int(ch["P"]) for ch in chains], np.int32)
    Ss = Ns + Ps
    # shared pair tables: one device block per distinct (distances, tc) pair of arrays
    blocks, key_of, pair_off = [], {}, np.zeros(n, np.int64)
    off = 0
    for c, ch in enumerate(chains):
        k = (id(ch["distances"]), id(ch["transitions_constant"]))
        if k not in key_of:
            key_of[k] = off
            blocks.append((np.asarray(ch["distances"], np.float64).reshape(-1),
                           np.asarray(ch["transitions_constant"], np.float64).reshape(-1)))
            off += int(Ss[c]) ** 2
        pair_off[c] = key_of[k]
    cat = lambda xs, dt: np.ascontiguousarray(np.concatenate([np.asarray(x, dt).reshape(-1) for x in xs]))  # noqa: E731
    site_off = np.concatenate([[0], np.cumsum(Ns)[:-1]]).astype(np.int64)
    se_off = np.concatenate([[0], np.cumsum(Ss)[:-1]]).astype(np.int64)
    el_off = np.concatenate([[0], np.cumsum(Ps)[:-1]]).astype(np.int64)
    tr_off = np.concatenate([[0], np.cumsum(Ss.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    smax = int(Ss.max())
    T = lambda a, dt: _dev(a, dt, d)  # noqa: E731
    keep = dict(
        N=T(Ns, torch.int32), P=T(Ps, torch.int32),
        nu=T([float(ch["nu"]) for ch in chains], f64), kT=T([float(ch["kT"]) for ch in chains], f64),
        I_0=T([float(ch["I_0"]) for ch in chains], f64), R=T([float(ch["R"]) for ch in chains], f64),
        pair_off=T(pair_off, i64), distances=T(cat([b[0] for b in blocks], np.float64), f64),
        tc=T(cat([b[1] for b in blocks], np.float64), f64),
        site_off=T(site_off, i64), Ec=T(cat([ch["E_constant"] for ch in chains], np.float64), f64),
        se_off=T(se_off, i64), se=T(cat([ch["site_energies"] for ch in chains], np.float64), f64),
        occ=T(cat([ch["occupation"] for ch in chains], np.uint8), torch.uint8),
        el_off=T(el_off, i64), eo=torch.zeros(max(int(Ps.sum()), 1), dtype=i64, device=d),
        hops=T(np.broadcast_to(np.asarray(hops, np.int64), (n,)), i64),
        seeds=T(np.asarray([int(s_) & (2**64 - 1) for s_ in seeds], np.uint64).view(np.int64), i64),
        t_out=torch.zeros(n, dtype=f64, device=d), s_out=torch.zeros(n, dtype=torch.int32, device=d))
    L = lib()
    wsb = L.kmc_simulate_f64_batch_workspace_size(n, smax)
    keep["ws"] = torch.empty(max(wsb, 8), dtype=torch.uint8, device=d)
    b = _native.KmcF64Batch()
    b.n_chains, b.max_sites, b.record = n, smax, int(bool(record))
    b.N, b.P = keep["N"].data_ptr(), keep["P"].data_ptr()
    b.nu, b.kT, b.I_0, b.R = (keep[k].data_ptr() for k in ("nu", "kT", "I_0", "R"))
    b.pair_off, b.distances, b.transitions_constant = (keep["pair_off"].data_ptr(), keep["distances"].data_ptr(),
                                                       keep["tc"].data_ptr())
    b.site_off, b.E_constant = keep["site_off"].data_ptr(), keep["Ec"].data_ptr()
    b.se_off, b.site_energies = keep["se_off"].data_ptr(), keep["se"].data_ptr()
    b.occupation, b.el_off, b.electrode_occupation = (keep["occ"].data_ptr(), keep["el_off"].data_ptr(),
                                                      keep["eo"].data_ptr())
    b.hops, b.seeds = keep["hops"].data_ptr(), keep["seeds"].data_ptr()
    if record:
        keep["tr_off"] = T(tr_off, i64)
        keep["tr"] = torch.zeros(max(int((Ss.astype(np.int64) ** 2).sum()), 1), dtype=f64, device=d)
        keep["oit"] = torch.zeros(max(int(Ns.sum()), 1), dtype=f64, device=d)
        b.traffic_off, b.traffic, b.occupations_in_time = (keep["tr_off"].data_ptr(), keep["tr"].data_ptr(),
                                                           keep["oit"].data_ptr())
    if flux:
        keep["fx"] = torch.zeros(max(int(Ps.sum()), 1), dtype=f64, device=d)
        b.flux_time = keep["fx"].data_ptr()
    b.time_out, b.status_out = keep["t_out"].data_ptr(), keep["s_out"].data_ptr()
    b.workspace, b.workspace_bytes = keep["ws"].data_ptr(), wsb
    check(L.kmc_simulate_f64_batch(C.byref(b), _stream_handle()))
    torch.cuda.synchronize(d)
    times = keep["t_out"].cpu().numpy()
    eo = keep["eo"].cpu().numpy()
    eos = [eo[o:o + p] for o, p in zip(el_off, Ps)]
    status = keep["s_out"].cpu().numpy()
    res = [times, eos, status]
    if record:
        oit = keep["oit"].cpu().numpy()
        res.append([oit[o:o + k] for o, k in zip(site_off, Ns)])
    if flux:
        fx = keep["fx"].cpu().numpy()
        res.append([fx[o:o + p] for o, p in zip(el_off, Ps)])
    return tuple(res)


# ---------------------------------------------------------------------------
# batched FP32 engine
# ---------------------------------------------------------------------------

@dataclass
class TableSpec:
    """One geometry instance: the FP64 tables the hop loop reads.

    ``positions`` (S, 3: acceptors then electrodes) and ``ab`` are needed for
    the positions pair mode, where the engine evaluates d_ij from the
    coordinates; that mode is only valid when ``distances`` and
    ``transitions_constant`` are the tables of those positions
    (calc_distances / calc_transitions_constant), which ``check_positions``
    verifies."""
    N: int
    P: int
    nu: float
    I_0: float
    R: float
    distances: np.ndarray
    transitions_constant: np.ndarray
    positions: Optional[np.ndarray] = None
    ab: Optional[float] = None
    from_positions: bool = False      # tables computed from `positions` by this package

    @property
    def S(self):
        return self.N + self.P

    @classmethod
    def from_network(cls, net):
        pos = np.concatenate([np.asarray(net.acceptors, np.float64).reshape(-1, 3),
                              np.asarray(net.electrodes, np.float64)[:, :3]], axis=0)
        return cls(net.N, net.P, float(net.nu), float(net.I_0), float(net.R), net.distances,
                   net.transitions_constant, pos, float(net.ab),
                   from_positions=bool(getattr(net, "tables_from_positions", True)))

    def check_positions(self, rtol=1e-9):
        """True when the tables are those of the positions."""
        if self.positions is None or self.ab is None:
            return False
        if self.from_positions:
            return True
        from . import geometry as geo
        d = geo.site_distances(self.positions[: self.N], np.concatenate(
            [self.positions[self.N:], np.zeros((self.P, 1))], axis=1))
        tc = geo.transitions_constant(d, self.nu, self.ab)
        return bool(np.allclose(d, self.distances, rtol=rtol, atol=0) and
                    np.allclose(tc, self.transitions_constant, rtol=rtol, atol=1e-300))


def default_lanes(S):
    """Threads per chain by size (the autotuner refines this per workload):
    warp slices for small networks, whole blocks for large ones."""
    if S <= 48:
        return 16
    if S <= 128:
        return 32
    if S <= 512:
        return 128
    return 256


_REANCHOR = 1024
LANE_CHOICES = (4, 8, 16, 32, 64, 128, 256, 512)


def balanced_warps_per_block(n_work, sms):
    """Warps per block for a warp-slice launch of n_work warp items: the size
    that puts the fewest warps on the busiest SM while every block is
    resident at once at 16 warps per SM (2048 items on 152 SMs: 7 warps, 293
    blocks, at most 14 warps on an SM, where 8 warps leave 104 SMs with 16
    and 48 with 8); 8 when no size fits in one wave.  The C host path uses
    the same rule."""
    best, best_load = 8, None
    for w in range(8, 3, -1):
        blocks = (n_work + w - 1) // w
        if blocks > (16 // w) * sms:
            continue
        load = ((blocks + sms - 1) // sms) * w
        if best_load is None or load < best_load:
            best, best_load = w, load
    return best


def widen_small_launch(G, S, n_chains, sms):
    """Lanes for a chain of a launch too small to fill the GPU: its run time
    is one chain's per-hop latency, so each chain gets a wider group (one
    N=120 chain: 2.7 us per hop at 256 lanes, 12.9 us at the size default of
    32), up to twice the next power of two of S and 512 lanes, while the
    launch's chains x lanes stay within a quarter of the engine's resident
    threads (512 per SM).  The C host path applies the same rule."""
    p = 1
    while p < S:
        p <<= 1
    target = min(512, 2 * p)
    budget = sms * 512 // 4
    while G < target and n_chains * 2 * G <= budget:
        G *= 2
    return G


def make_work_lists(S_c, hops, lanes=None, sms=None):
    """Bin chains by lanes-per-chain and pack each bin into warp items.

    Returns a list of (G, work, order, max_sites): ``work`` holds 32/G chain
    ids per warp item (-1 pads the last item).  Where a warp item holds
    several chains they are ordered by size, then hop budget (both
    descending), so that the chains sharing a warp have similar per-hop work
    and similar lifetimes; where an item is one chain (G >= 32) they are
    ordered by their work, hops x S^2, longest first, so that the longest
    chains start in the first wave of blocks instead of setting the end of
    the launch from a later one.  With lanes None the size default applies,
    widened for a launch too small to fill the GPU when the device's SM
    count ``sms`` is given (``widen_small_launch``)."""
    S_c = np.asarray(S_c, np.int64).reshape(-1)
    hops = np.broadcast_to(np.asarray(hops, np.int64), S_c.shape)
    if lanes is None:
        n = S_c.shape[0]
        lane_of = np.array([default_lanes(int(s)) if sms is None else
                            widen_small_launch(default_lanes(int(s)), int(s), n, sms) for s in S_c], np.int32)
    elif callable(lanes):
        lane_of = np.array([int(lanes(int(s))) for s in S_c], np.int32)
    else:
        lane_of = np.full(S_c.shape[0], int(lanes), np.int32)
    bad = set(lane_of.tolist()) - set(LANE_CHOICES)
    if bad:
        raise ValueError(f"lanes per chain must be one of {LANE_CHOICES}, got {sorted(bad)}")
    out = []
    for G in sorted(set(lane_of.tolist())):
        idx = np.flatnonzero(lane_of == G)
        cpw = max(1, 32 // G)
        if cpw == 1:
            work_est = hops[idx].astype(np.float64) * S_c[idx].astype(np.float64) ** 2
            order = idx[np.lexsort((-hops[idx], -S_c[idx], -work_est))]
        else:
            order = idx[np.lexsort((-hops[idx], -S_c[idx]))]
        nw = (len(order) + cpw - 1) // cpw
        work = np.full(nw * cpw, -1, np.int32)
        work[: len(order)] = order
        out.append((int(G), work, order, int(S_c[idx].max())))
    return out


class TableSet:
    """Device-resident geometry data, built once and shared by batches:
    FP32 pair tables (L, B) from the FP64 tables (kmc_build_table) and, in
    positions mode, the site coordinates and rate constants."""

    def __init__(self, specs: Sequence[TableSpec], pair_mode="table", dev=None):
        d = device(dev)
        self.specs = list(specs)
        Ns = np.array([t.N for t in self.specs], np.int32)
        Ps = np.array([t.P for t in self.specs], np.int32)
        if np.any(Ps > 64):
            raise ValueError("the engine supports at most 64 electrodes")
        if pair_mode not in ("table", "positions"):
            raise ValueError("pair_mode must be 'table' or 'positions'")
        tab_off = np.zeros(len(self.specs), np.int64)
        off = 0
        build = pair_mode == "table"          # positions mode never reads the pair tables
        for i, t in enumerate(self.specs):
            tab_off[i] = off
            off += 2 * t.S * t.S if build else 0
        self.tab_LB = torch.empty(max(off, 2), dtype=torch.float32, device=d)
        L = lib()
        sh = _stream_handle()
        for i, t in enumerate(self.specs if build else []):
            dd = _dev(np.asarray(t.distances, np.float64).reshape(t.S, t.S), torch.float64, d)
            tc = _dev(np.asarray(t.transitions_constant, np.float64).reshape(t.S, t.S), torch.float64, d)
            check(L.kmc_build_table(t.N, t.P, float(t.nu), float(t.I_0), float(t.R), _ptr(dd), _ptr(tc),
                                    C.c_void_p(self.tab_LB.data_ptr() + 4 * int(tab_off[i])), sh))
            torch.cuda.current_stream().synchronize()
        self.tab_N = _dev(Ns, torch.int32, d)
        self.tab_P = _dev(Ps, torch.int32, d)
        self.tab_off = _dev(tab_off, torch.int64, d)
        self.pair_mode = _native.PAIRS_POSITIONS if pair_mode == "positions" else _native.PAIRS_TABLE
        self.tab_pos = self.tab_pos_off = self.tab_coef = None
        if pair_mode == "positions":
            pos_off = np.zeros(len(self.specs), np.int64)
            rows, coef, off = [], [], 0
            for i, t in enumerate(self.specs):
                if not t.check_positions():
                    raise ValueError(f"table {i}: positions mode needs tables computed from its positions")
                p4 = np.zeros((t.S, 4), np.float32)
                p4[:, :3] = t.positions
                rows.append(p4.reshape(-1))
                pos_off[i] = off
                off += 4 * t.S
                coef.append([-2.0 * np.log2(np.e) / t.ab, np.log2(t.nu * t.nu), t.I_0 * t.R, 0.0])
            self.tab_pos = _dev(np.concatenate(rows), torch.float32, d)
            self.tab_pos_off = _dev(pos_off, torch.int64, d)
            self.tab_coef = _dev(np.asarray(coef, np.float32).reshape(-1), torch.float32, d)


class Batch:
    """Device-resident chains for the batched FP32 engine.

    tables:      list of TableSpec (or a prebuilt TableSet); chains name one
                 by index.
    chain_table: (C,) table index per chain.
    kT:          (C,) temperature per chain.
    E_constant:  list of (N_c,) arrays, or a (C, N) array when all chains
                 share N; alternatively pass ``E_constant_dev`` (a float32
                 CUDA tensor pool) produced by ``superpose``.
    el_energy:   list of (P_c,) electrode energies, or (C, P).
    occupation:  list/array of initial occupations.
    hops:        (C,) hop budget per chain.
    streams:     (C,) RNG stream ids (default: chain index); seed keys them.
    record:      _native.RECORD_NONE / RECORD_NUMBA / RECORD_GO.
    lanes:       None (by size class), an int for every chain, or a callable
                 S -> lanes.
    warps_per_block: warps per block of the warp-slice launches: an int, a
                 dict or callable of the lanes per chain (as the autotuner
                 returns them), or None for the balanced size of each bin
                 (``balanced_warps_per_block``).
    """

    def __init__(self, tables, chain_table, kT, E_constant=None,
                 el_energy=None, occupation=None, hops=None, *, streams=None, seed=0,
                 record=_native.RECORD_NONE, lanes=None, warps_per_block=None, dev=None,
                 replay=None, E_constant_dev=None, el_energy_dev=None, reanchor=_REANCHOR,
                 pair_mode="table", hop_log=False, hop_rates=False, count_select_mismatch=False,
                 measure_drift=False, persistent=False, flux=False):
        self.dev = device(dev)
        d = self.dev
        tables_set = tables if isinstance(tables, TableSet) else None
        self.tables = list(tables.specs) if tables_set is not None else list(tables)
        ct = np.asarray(chain_table, np.int32).reshape(-1)
        self.n = n = ct.shape[0]
        self.chain_table = ct
        Ns = np.array([t.N for t in self.tables], np.int32)
        Ps = np.array([t.P for t in self.tables], np.int32)
        if np.any(Ps > 64):
            raise ValueError("the engine supports at most 64 electrodes")
        self.N_c = Ns[ct]
        self.P_c = Ps[ct]
        self.S_c = self.N_c + self.P_c
        self.record = int(record)
        self.seed = int(seed) & (2**64 - 1)
        self.reanchor = int(reanchor)
        # warps per block of the warp-slice launches: one value, or per lanes
        # width (a dict G -> warps, or a callable G -> warps, as the
        # autotuner returns it)
        self.warps_per_block = warps_per_block
        self._sms = torch.cuda.get_device_properties(d).multi_processor_count

        ts = tables_set if tables_set is not None else TableSet(self.tables, pair_mode=pair_mode, dev=d)
        self.table_set = ts
        self.tab_N, self.tab_P, self.tab_off, self.tab_LB = ts.tab_N, ts.tab_P, ts.tab_off, ts.tab_LB
        self.pair_mode = ts.pair_mode
        self.tab_pos, self.tab_pos_off, self.tab_coef = ts.tab_pos, ts.tab_pos_off, ts.tab_coef

        # per-chain offsets
        self.site_off = np.concatenate([[0], np.cumsum(self.N_c)[:-1]]).astype(np.int64)
        self.el_off = np.concatenate([[0], np.cumsum(self.P_c)[:-1]]).astype(np.int64)
        self.pair_off = np.concatenate([[0], np.cumsum(self.S_c.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
        nsite = int(self.N_c.sum())
        nel = int(self.P_c.sum())

        def pool(vals, total, dtype, np_dtype):
            if isinstance(vals, np.ndarray) and vals.ndim == 2:
                flat = vals.astype(np_dtype).reshape(-1)
            else:
                flat = np.concatenate([np.asarray(v, np_dtype).reshape(-1) for v in vals]) if total else np.zeros(0, np_dtype)
            if flat.shape[0] != total:
                raise ValueError(f"pool size {flat.shape[0]} != {total}")
            return _dev(flat if total else np.zeros(1, np_dtype), dtype, d)

        self.E_constant = E_constant_dev if E_constant_dev is not None else pool(E_constant, nsite, torch.float32, np.float32)
        self.el_energy = el_energy_dev if el_energy_dev is not None else pool(el_energy, nel, torch.float32, np.float32)
        self.occupation = pool(occupation, nsite, torch.uint8, np.uint8)
        self.chain_tab_d = _dev(ct, torch.int32, d)
        kT32 = np.broadcast_to(np.asarray(kT, np.float32), (n,))
        self.kT = _dev(kT32, torch.float32, d)
        # one temperature for every chain: the engine may fold it into a staged table
        self.uniform_kT = float(kT32[0]) if n and np.all(kT32 == kT32[0]) else 0.0
        self.site_off_d = _dev(self.site_off, torch.int64, d)
        self.el_off_d = _dev(self.el_off, torch.int64, d)
        self.pair_off_d = _dev(self.pair_off, torch.int64, d)
        self.electrode_occupation = torch.zeros(max(nel, 1), dtype=torch.int64, device=d)
        self.time = torch.zeros(n, dtype=torch.float64, device=d)
        self.hops_done = torch.zeros(n, dtype=torch.int64, device=d)
        self.hops_total = _dev(np.broadcast_to(np.asarray(hops, np.int64), (n,)), torch.int64, d)
        sid = np.arange(n, dtype=np.uint64) if streams is None else np.asarray(streams, np.uint64)
        self.stream_ids = _dev(sid.view(np.int64), torch.int64, d)
        self.status = torch.zeros(n, dtype=torch.int32, device=d)
        self.n_pairs = torch.zeros(n, dtype=torch.int64, device=d)
        if self.record:
            self.occ_time = torch.zeros(max(nsite, 1), dtype=torch.float64, device=d)
            self.occ_since = torch.zeros(max(nsite, 1), dtype=torch.float64, device=d)
            self.traffic = torch.zeros(max(int((self.S_c.astype(np.int64) ** 2).sum()), 1),
                                       dtype=torch.int32, device=d)
        else:
            self.occ_time = self.occ_since = self.traffic = None
        self.replay = self.replay_off = None
        if replay is not None:
            rows = [np.asarray(r, np.float64).reshape(-1) for r in replay]
            need = 2 * np.broadcast_to(np.asarray(hops, np.int64), (n,))
            if len(rows) != n or any(r.shape[0] < k for r, k in zip(rows, need)):
                raise ValueError("replay needs one stream of at least 2*hops uniforms per chain")
            roff = np.concatenate([[0], np.cumsum([r.shape[0] for r in rows])[:-1]]).astype(np.int64)
            self.replay = _dev(np.concatenate(rows), torch.float64, d)
            self.replay_off = _dev(roff, torch.int64, d)
        # optional per-hop log: (from, to) and (total rate, chosen pair's rate)
        # of every hop, hops_total entries per chain
        self.hop_log = self.hop_rates = self.hop_log_off = None
        if hop_log or hop_rates:
            ht = np.broadcast_to(np.asarray(hops, np.int64), (n,))
            self._log_off = np.concatenate([[0], np.cumsum(ht)[:-1]]).astype(np.int64)
            total = int(ht.sum())
            self.hop_log = torch.full((max(2 * total, 2),), -1, dtype=torch.int32, device=d)
            if hop_rates:
                self.hop_rates = torch.zeros(max(2 * total, 2), dtype=torch.float32, device=d)
            self.hop_log_off = _dev(self._log_off, torch.int64, d)
        # debug builds: per chain, hops an FP64 selection would pick differently
        self.select_mismatch = (torch.zeros(n, dtype=torch.int64, device=d)
                                if count_select_mismatch else None)
        # electrode pool: time integral of each electrode's expected net inflow
        self.flux_time = torch.zeros(max(nel, 1), dtype=torch.float64, device=d) if flux else None
        # per chain: largest incremental-energy drift found at a re-anchor (kT)
        self.energy_drift = torch.zeros(n, dtype=torch.float32, device=d) if measure_drift else None
        self.cancel = None            # a CancelWord, or None
        self.time_budget_ns = 0       # per launch and chain; 0: none
        self._bins = self._make_bins(lanes, np.broadcast_to(np.asarray(hops, np.int64), (n,)))
        # persistent launches: one work counter per bin, zeroed before each launch
        self.persistent = bool(persistent)
        self._counters = (torch.zeros(max(len(self._bins), 1), dtype=torch.int32, device=d)
                          if self.persistent else None)

    def _warps(self, G, n_work=None):
        w = self.warps_per_block
        if w is None:
            return balanced_warps_per_block(n_work, self._sms) if n_work is not None and G <= 32 else 8
        if callable(w):
            w = w(G)
        elif isinstance(w, dict):
            w = w.get(G, 4)
        return int(w) if w else 4

    # -- work lists --------------------------------------------------------
    def _make_bins(self, lanes, hops):
        bins = []
        for G, work, order, smax in make_work_lists(self.S_c, hops, lanes, sms=self._sms):
            bins.append(dict(G=G, n_work=len(work) // max(1, 32 // G), work=_dev(work, torch.int32, self.dev),
                             max_sites=smax, chains=order))
        return bins

    def _struct(self, bin_, seg):
        b = _native.KmcBatch()
        b.n_tables = len(self.tables)
        b.max_sites = bin_["max_sites"]
        b.tab_N, b.tab_P, b.tab_off, b.tab_LB = (self.tab_N.data_ptr(), self.tab_P.data_ptr(),
                                                 self.tab_off.data_ptr(), self.tab_LB.data_ptr())
        b.n_chains = self.n
        b.lanes_per_chain = bin_["G"]
        b.chain_tab = self.chain_tab_d.data_ptr()
        b.chain_kT = self.kT.data_ptr()
        b.chain_site_off = self.site_off_d.data_ptr()
        b.chain_el_off = self.el_off_d.data_ptr()
        b.chain_pair_off = self.pair_off_d.data_ptr()
        b.E_constant = self.E_constant.data_ptr()
        b.el_energy = self.el_energy.data_ptr()
        b.occupation = self.occupation.data_ptr()
        b.electrode_occupation = self.electrode_occupation.data_ptr()
        b.time = self.time.data_ptr()
        b.hops_done = self.hops_done.data_ptr()
        b.hops_total = self.hops_total.data_ptr()
        b.stream = self.stream_ids.data_ptr()
        b.status = self.status.data_ptr()
        b.n_pairs = self.n_pairs.data_ptr()
        if self.record:
            b.occ_time, b.occ_since, b.traffic = (self.occ_time.data_ptr(), self.occ_since.data_ptr(),
                                                  self.traffic.data_ptr())
        b.work = bin_["work"].data_ptr()
        b.n_work = bin_["n_work"]
        b.record = self.record
        b.reanchor = self.reanchor
        b.warps_per_block = self._warps(bin_["G"], bin_["n_work"])
        b.max_hops_per_launch = int(seg)
        b.seed = self.seed
        if self.replay is not None:
            b.replay, b.replay_off = self.replay.data_ptr(), self.replay_off.data_ptr()
        if self.cancel is not None:
            b.cancel = self.cancel.device
        b.time_budget_ns = int(self.time_budget_ns)
        b.uniform_kT = self.uniform_kT
        if self.select_mismatch is not None:
            b.select_mismatch = self.select_mismatch.data_ptr()
        if self.energy_drift is not None:
            b.energy_drift = self.energy_drift.data_ptr()
        if self.flux_time is not None:
            b.flux_time = self.flux_time.data_ptr()
        if self.hop_log is not None:
            b.hop_log, b.hop_log_off = self.hop_log.data_ptr(), self.hop_log_off.data_ptr()
            if self.hop_rates is not None:
                b.hop_rates = self.hop_rates.data_ptr()
        b.pair_mode = self.pair_mode
        if self.tab_pos is not None:
            b.tab_pos, b.tab_pos_off, b.tab_coef = (self.tab_pos.data_ptr(), self.tab_pos_off.data_ptr(),
                                                    self.tab_coef.data_ptr())
        return b

    def launch(self, max_hops_per_launch=None, stream=None, bin_streams=None):
        """One launch per size bin: advance every chain by up to
        max_hops_per_launch hops (a multiple of the re-anchor period).  Bins
        go to `stream`, or round-robin to `bin_streams` so that launches of
        different sizes run side by side (the caller synchronises)."""
        seg = max_hops_per_launch
        if seg is None:
            seg = int(self.hops_total.max().item()) if self.n else 1
        seg = max(self.reanchor, ((int(seg) + self.reanchor - 1) // self.reanchor) * self.reanchor)
        L = lib()
        for i, bin_ in enumerate(self._bins):
            st = bin_streams[i % len(bin_streams)] if bin_streams else stream
            b = self._struct(bin_, seg)
            if self._counters is not None:
                ctr = self._counters[i:i + 1]
                with torch.cuda.stream(st if st is not None else torch.cuda.current_stream()):
                    ctr.zero_()
                b.work_counter = ctr.data_ptr()
            check(L.kmc_run_batch(C.byref(b), _stream_handle(st)))
        return self

    def run(self, stream=None):
        self.launch(None, stream)
        return self

    def results(self, stream=None):
        """Copy results to the host: dict of numpy arrays (ragged per chain
        lists for occupations and electrode counts).  With `stream`, wait for
        that stream only (the one this batch was launched on) and copy on it;
        otherwise synchronise the device."""
        if stream is not None:
            with torch.cuda.stream(stream):
                stream.synchronize()
                return self._results()
        torch.cuda.synchronize(self.dev)
        return self._results()

    def _results(self):
        eo = self.electrode_occupation.cpu().numpy()
        occ = self.occupation.cpu().numpy()
        out = dict(time=self.time.cpu().numpy(), status=self.status.cpu().numpy(),
                   hops_done=self.hops_done.cpu().numpy(), n_pairs=self.n_pairs.cpu().numpy())
        out["electrode_occupation"] = [eo[o:o + p] for o, p in zip(self.el_off, self.P_c)]
        out["occupation"] = [occ[o:o + n].astype(bool) for o, n in zip(self.site_off, self.N_c)]
        if self.select_mismatch is not None:
            out["select_mismatch"] = self.select_mismatch.cpu().numpy()
        if self.energy_drift is not None:
            out["energy_drift"] = self.energy_drift.cpu().numpy()
        if self.flux_time is not None:
            ft = self.flux_time.cpu().numpy()
            out["flux_time"] = [ft[o:o + p] for o, p in zip(self.el_off, self.P_c)]
        if self.hop_log is not None:
            ht = self.hops_total.cpu().numpy()
            lg = self.hop_log.cpu().numpy()
            out["hop_log"] = [lg[2 * o:2 * (o + k)].reshape(k, 2) for o, k in zip(self._log_off, ht)]
            if self.hop_rates is not None:
                hr = self.hop_rates.cpu().numpy()
                out["hop_rates"] = [hr[2 * o:2 * (o + k)].reshape(k, 2) for o, k in zip(self._log_off, ht)]
        if self.record:
            ot = self.occ_time.cpu().numpy()
            tr = self.traffic.cpu().numpy()
            out["occ_time"] = [ot[o:o + n] for o, n in zip(self.site_off, self.N_c)]
            out["traffic"] = [tr[o:o + s * s].reshape(s, s) for o, s in zip(self.pair_off, self.S_c)]
        return out

    def currents(self):
        """electrode_occupation / time per chain, as (C, P) when P is uniform."""
        r = self.results()
        cur = [e / t if t > 0 else np.full(e.shape, np.nan) for e, t in zip(r["electrode_occupation"], r["time"])]
        if len(set(self.P_c.tolist())) == 1:
            return np.array(cur)
        return cur


def superpose(basis, comp, voltages, mu=0.0, dev=None, stream=None):
    """Constant site energies of many chains on one geometry, on the device:
    returns (E_constant float32 (C*N,), el_energy float32 (C*P,))."""
    d = device(dev)
    basis = np.asarray(basis, np.float64)
    V = np.asarray(voltages, np.float64)
    C_, P = V.shape
    N = basis.shape[1]
    b = _dev(basis, torch.float64, d)
    v = _dev(V, torch.float64, d)
    cp = _dev(np.asarray(comp, np.float64), torch.float64, d)
    ec = torch.empty(max(C_ * N, 1), dtype=torch.float32, device=d)
    ve = torch.empty(max(C_ * P, 1), dtype=torch.float32, device=d)
    check(lib().kmc_site_energies(C_, N, P, _ptr(b), _ptr(v), float(mu), _ptr(cp), _ptr(ec), _ptr(ve),
                                  _stream_handle(stream)))
    return ec, ve


# ---------------------------------------------------------------------------
# keyword-compatible replacement for the reference's hop-loop functions
# ---------------------------------------------------------------------------

def simulate_cuda(N_acceptors, N_electrodes, nu, kT, I_0, R, time, occupation, distances,
                  E_constant, site_energies, transitions_constant, transitions=None,
                  problist=None, electrode_occupation=None, hops=100000, record=False,
                  goSpecificFunction=None, prune_threshold=0.0, precision="fp32", seed=None,
                  record_convention="numba", lanes=None):
    """Drop-in for ``_simulate_discrete_record(**args)`` (and for
    ``callGoSimulation`` when called with ``goSpecificFunction``) inside
    ``kmc_dn.makeSimulation`` (kmc_dopant_networks.py:544-619).

    Returns ``(time, occupation, electrode_occupation, traffic,
    occupations_in_time)``; ``occupation`` is the final state and
    ``electrode_occupation`` the per-electrode hole count of this run.
    precision "fp64" runs the plain FP64 kernel (the numba loop's
    arithmetic), "fp32" the batched engine with one chain."""
    N, P = int(N_acceptors), int(N_electrodes)
    hops = int(hops)
    if seed is None:
        seed = int(np.random.randint(0, 2**63 - 1, dtype=np.int64))
    occ0 = np.asarray(occupation, dtype=bool).reshape(N)
    if precision == "fp64":
        r = simulate_f64(N, P, nu, kT, I_0, R, occ0, distances, E_constant, site_energies,
                         transitions_constant, hops, record=record, seed=seed)
        if r["status"] != 0:
            raise _native.KmcError(r["status"], "hop loop stopped: no allowed transition or non-finite total rate")
        return (r["time"], r["occupation"], r["electrode_occupation"], r["traffic"],
                r["occupations_in_time"])
    if precision != "fp32":
        raise ValueError("precision must be 'fp32' or 'fp64'")
    S = N + P
    spec = TableSpec(N, P, float(nu), float(I_0), float(R), np.asarray(distances, np.float64),
                     np.asarray(transitions_constant, np.float64))
    rec = 0
    if record:
        rec = _native.RECORD_GO if record_convention == "go" else _native.RECORD_NUMBA
    se = np.asarray(site_energies, np.float64).reshape(S)
    b = Batch([spec], [0], [float(kT)], [np.asarray(E_constant, np.float64)], [se[N:]], [occ0.astype(np.uint8)],
              [hops], seed=seed, record=rec, lanes=lanes)
    b.run()
    r = b.results()
    if r["status"][0] != 0:
        raise _native.KmcError(int(r["status"][0]), "hop loop stopped: no allowed transition or non-finite total rate")
    traffic = r["traffic"][0].astype(np.float64) if record else np.zeros((S, S))
    oit = r["occ_time"][0] if record else np.zeros(N)
    return (float(r["time"][0]), r["occupation"][0], r["electrode_occupation"][0].astype(np.int64),
            traffic, oit)


def prune(transitions_constant, threshold):
    """Zero the pairs a pruned Go run leaves out of its transition list: it
    keeps ``tc > threshold * max(tc)`` (simulation.go:199-215), all in
    float32 as the Go code holds them (the product rounded to float32 before
    the compare).  A zero constant gives a zero rate, so a pruned pair can
    never be selected."""
    tc = np.array(transitions_constant, dtype=np.float64, copy=True)
    if threshold and threshold > 0:
        t32 = tc.astype(np.float32)
        cut = np.float32(np.float32(threshold) * np.float32(t32.max()))
        tc[~(t32 > cut)] = 0.0
    return tc


def simulate_go(N_acceptors, N_electrodes, nu, kT, I_0, R, time, occupation, distances,
                E_constant, site_energies, transitions_constant, transitions=None, problist=None,
                electrode_occupation=None, hops=100000, record=False,
                goSpecificFunction="wrapperSimulateRecord", prune_threshold=0.0, seed=None,
                lanes=None):
    """Drop-in for ``callGoSimulation`` (goSimulation/pythonBind.py:49-92)
    with the Go library's semantics on the FP32 engine: the chain starts with
    every acceptor empty (simulationWrapper.go:134-141), the caller's
    occupation comes back unchanged (pythonBind.py:84), record counts net
    traffic and credits occupancy before each hop (simulation.go:309-317).
    ``goSpecificFunction="wrapperSimulateProbability"`` runs the mean-field
    relaxation instead (``meanfield.simulate_probability``).  Returns (time,
    occupation, electrode_occupation[, traffic, average_occupation])."""
    if goSpecificFunction == "wrapperSimulateProbability":
        from .meanfield import simulate_probability
        return simulate_probability(N_acceptors, N_electrodes, nu, kT, I_0, R, time, occupation,
                                    distances, E_constant, site_energies, transitions_constant,
                                    hops=hops, record=record)
    N, P = int(N_acceptors), int(N_electrodes)
    if seed is None:
        seed = int(np.random.randint(0, 2**63 - 1, dtype=np.int64))
    thr = prune_threshold if goSpecificFunction == "wrapperSimulatePruned" else 0.0
    tc = prune(transitions_constant, thr)
    S = N + P
    se = np.asarray(site_energies, np.float64).reshape(S)
    spec = TableSpec(N, P, float(nu), float(I_0), float(R), np.asarray(distances, np.float64), tc)
    b = Batch([spec], [0], [float(kT)], [np.asarray(E_constant, np.float64)], [se[N:]],
              [np.zeros(N, np.uint8)], [int(hops)], seed=seed,
              record=_native.RECORD_GO if record else _native.RECORD_NONE, lanes=lanes)
    r = b.run().results()
    if r["status"][0] != 0:
        raise _native.KmcError(int(r["status"][0]), "hop loop stopped: no allowed transition or non-finite total rate")
    occ_out = np.array([int(x) for x in np.asarray(occupation).reshape(N)])
    eo = r["electrode_occupation"][0].astype(np.int64)
    if not record:
        return float(r["time"][0]), occ_out, eo
    return (float(r["time"][0]), occ_out, eo, r["traffic"][0].astype(np.float64), r["occ_time"][0])
