"""Benchmark: hops/s of the batched FP32 engine on the homogeneous ensemble.

Workload (one step): 4096 independent chains on the N=30, M=3, 20x20,
8-electrode network (kmc_dn_gb300.workloads.plain_network), each chain with
its own U[-1,1] voltage vector and RNG stream, 1e6 hops per chain, run as
one graph-captured launch of the engine.  Inputs are synthetic and seeded
(the reference publishes no dataset for this path).

Printed (rank 0, one JSON line): whole-job hops/s with inputs resident on
the device (`value`), the same through the host-buffer C entry point
(`e2e`), the plain single-chain FP64 kernel's hops/s on the same network
(`fp64_single_chain`), the roofline of the dominant kernel against the
measured ex2 (SFU) rate, the CPU baseline (the C restatement of the
reference's Go loop on host threads), and SM clocks sampled during the
timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

For N > 1 (torchrun, one rank per GPU) every rank runs its own 4096 chains
(weak scaling, no collective on the data path); time is the max over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N_CHAINS = 4096
HOPS = 1_000_000
METRIC = "hops/s on 1 GB300: batched FP32 vs plain FP64 at ≤1% current error; p99 lat"
WORKLOAD = "homogeneous ensemble: 4096 chains x 1e6 hops, N=30 M=3 P=8, 20x20, FP32 rates / FP64 clock"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(seed, n_chains, chain_offset=0):
    from kmc_dn_gb300 import workloads
    net, V = workloads.homogeneous_ensemble(n_chains + chain_offset, seed)
    return net, V[chain_offset:chain_offset + n_chains]


def cpu_baseline(net, V, threads, hops, n_chains, budget_s=20.0):
    """The C restatement of the reference's Go hop loop (no state memo),
    FP32 rates, O(N) energy updates, FP64 clock, one chain per host thread
    task, on a bounded sample of the workload's chains."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as orc
    N, P = net.N, net.P
    occ = np.tile(net.occupation.astype(np.uint8), (n_chains, 1))
    ec = np.stack([net.E_constant(v) for v in V[:n_chains]])
    se = np.stack([np.concatenate([np.zeros(N), v]) for v in V[:n_chains]])
    # calibrate: one short run to size the sample near budget_s
    t0 = time.perf_counter()
    orc.go_chains(N, P, net.nu, net.kT, net.I_0, net.R, occ[:threads], net.distances, ec[:threads],
                  se[:threads], net.transitions_constant, 2000, seed=7, threads=threads)
    per_hop = (time.perf_counter() - t0) / (2000 * threads) * threads   # s per hop per thread
    h = int(min(hops, max(2000, budget_s / max(per_hop, 1e-9) * threads / n_chains)))
    t0 = time.perf_counter()
    times, eo, na = orc.go_chains(N, P, net.nu, net.kT, net.I_0, net.R, occ, net.distances, ec, se,
                                  net.transitions_constant, h, seed=11, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": n_chains * h / dt, "unit": "hops/s", "cores": threads, "kind": "port",
            "sample": f"{n_chains} chains x {h} hops of the workload (C restatement of the "
                      f"reference's Go simulate loop, no memo), {dt:.1f} s wall"}


FLOOR = 0.05     # currents held to the 1 % level: |I| >= 5 % of the voltage vector's largest |I|


def _current_stats(I32, I64):
    """Per current: difference of the means, its standard error, z-score,
    relative difference and 3-sigma relative upper bound."""
    m32, m64 = I32.mean(0), I64.mean(0)
    se = np.sqrt(I32.var(0, ddof=1) / len(I32) + I64.var(0, ddof=1) / len(I64))
    d = np.abs(m32 - m64)
    den = np.maximum(np.abs(m64), 1e-300)
    return m64, se, d / np.maximum(se, 1e-300), d / den, (d + 3.0 * se) / den


def _summary(z, rel, up, ab):
    return {"max_abs_z": float(z.max()), "frac_within_3sigma": float(np.mean(z <= 3.0)),
            "resolved_within_1pct_at_3sigma": int(np.sum(ab & (up <= 0.01))),
            "point_estimate_within_1pct": int(np.sum(ab & (rel <= 0.01))),
            "max_rel_diff_above_floor": float(rel[ab].max()),
            "median_rel_diff_above_floor": float(np.median(rel[ab])),
            "max_rel_upper3_above_floor": float(up[ab].max()),
            "median_rel_upper3_above_floor": float(np.median(up[ab]))}


def accuracy_of(cases, dev, replicas32=512, replicas64=128, hops=300_000, seed=0, pair_mode="table"):
    """Electrode currents and occupations of the FP32 engine against the
    plain FP64 kernel (whose hop sequences equal the reference loop's, bit
    for bit), on independent replicas of each case.

    ``cases``: (network, voltages) pairs.  The FP32 chains take their
    constant site energies from the device superposition (kmc_site_energies,
    the path the timed workloads use); the FP64 chains take the host's FP64
    E_constant (the reference's set-up arithmetic).

    Two estimates of each current per chain: the count one, electrode
    hops / time (what the reference reports), and a control-variate one,
    count - beta * (count - flux) / time, where flux is the time integral of
    the electrode's expected net inflow (flux_time): count - flux is a
    zero-mean martingale, so any beta keeps the estimate unbiased, and beta
    (fitted per current on both sides' pooled within-side deviations, the
    same beta for both) removes the hop-by-hop Poisson noise the count
    carries.  Per current: the z-score of the difference of the means and,
    for every current above the magnitude floor (FLOOR of the vector's
    largest current), the relative difference and its 3-sigma upper bound
    (|dI| + 3 SE) / |I_FP64|; such a current is resolved at the 1 % level
    when that bound is <= 1 %.  Per site the time-averaged occupation
    likewise (z-score and absolute difference; both kernels credit
    occupancy after the hop)."""
    import torch
    from kmc_dn_gb300 import _native
    from kmc_dn_gb300.engine import Batch, TableSpec, simulate_f64_many, superpose
    rows = [c for c in range(len(cases)) for _ in range(replicas32)]
    specs = [TableSpec.from_network(net) if pair_mode == "positions" else
             TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
             for net, _ in cases]
    ec_parts, ve_parts = [], []
    for net, v in cases:
        ec, ve = superpose(net.basis, net.comp, np.tile(np.asarray(v, np.float64), (replicas32, 1)), net.mu, dev=dev)
        ec_parts.append(ec[:replicas32 * net.N])
        ve_parts.append(ve[:replicas32 * net.P])
    b = Batch(specs, np.array(rows, np.int32), [cases[c][0].kT for c in rows], None, None,
              [cases[c][0].occupation.astype(np.uint8) for c in rows], np.full(len(rows), hops),
              streams=np.arange(len(rows)) + 10_000_000, seed=seed + 101, dev=dev, pair_mode=pair_mode,
              record=_native.RECORD_NUMBA, E_constant_dev=torch.cat(ec_parts), el_energy_dev=torch.cat(ve_parts),
              flux=True)
    t0 = time.perf_counter()
    r32 = b.run().results()
    t32 = time.perf_counter() - t0
    assert np.all(r32["status"] == 0)
    rows64 = [c for c in range(len(cases)) for _ in range(replicas64)]
    chains = [dict(N=n.N, P=n.P, nu=n.nu, kT=n.kT, I_0=n.I_0, R=n.R, occupation=n.occupation,
                   distances=n.distances, E_constant=n.E_constant(v), site_energies=n.site_energies(v),
                   transitions_constant=n.transitions_constant) for n, v in (cases[c] for c in rows64)]
    t0 = time.perf_counter()
    t64, eo64, st64, oit64, fx64 = simulate_f64_many(
        chains, hops, [seed * 7919 + 13 + i for i in range(len(rows64))], dev=dev, record=True, flux=True)
    tf64 = time.perf_counter() - t0
    assert np.all(st64 == 0)
    cnt, cv, above, betas, vr, ozs, odiff = {"z": [], "rel": [], "up": []}, {"z": [], "rel": [], "up": []}, [], [], [], [], []
    per_current = []
    for c in range(len(cases)):
        i32 = [i for i, rc in enumerate(rows) if rc == c]
        i64 = [i for i, rc in enumerate(rows64) if rc == c]
        T32 = np.array([r32["time"][i] for i in i32])[:, None]
        T64 = np.array([t64[i] for i in i64])[:, None]
        C32 = np.stack([r32["electrode_occupation"][i] for i in i32]) / T32
        C64 = np.stack([eo64[i] for i in i64]) / T64
        D32 = C32 - np.stack([r32["flux_time"][i] for i in i32]) / T32
        D64 = C64 - np.stack([fx64[i] for i in i64]) / T64
        # beta per current from the pooled within-side deviations
        dc = np.concatenate([C32 - C32.mean(0), C64 - C64.mean(0)])
        dd = np.concatenate([D32 - D32.mean(0), D64 - D64.mean(0)])
        beta = (dc * dd).sum(0) / np.maximum((dd * dd).sum(0), 1e-300)
        betas.append(beta)
        m64, se_c, z, rel, up = _current_stats(C32, C64)
        cnt["z"].append(z), cnt["rel"].append(rel), cnt["up"].append(up)
        _, se_v, z, rel, up = _current_stats(C32 - beta * D32, C64 - beta * D64)
        cv["z"].append(z), cv["rel"].append(rel), cv["up"].append(up)
        per_current.extend([c, e, float(m64[e]), round(float(rel[e]), 5), round(float(up[e]), 5)]
                           for e in range(len(m64)) if abs(m64[e]) >= FLOOR * np.abs(m64).max())
        vr.append((se_c / np.maximum(se_v, 1e-300)) ** 2)
        above.append(np.abs(m64) >= FLOOR * np.abs(m64).max())
        O32 = np.stack([r32["occ_time"][i] / r32["time"][i] for i in i32])
        O64 = np.stack([oit64[i] / t64[i] for i in i64])
        osd = np.sqrt(O32.var(0, ddof=1) / len(i32) + O64.var(0, ddof=1) / len(i64))
        od = np.abs(O32.mean(0) - O64.mean(0))
        ozs.append(od / np.maximum(osd, 1e-12))
        odiff.append(od)
    ab = np.concatenate(above)
    cat = {k: np.concatenate(v) for k, v in cnt.items()}
    catv = {k: np.concatenate(v) for k, v in cv.items()}
    oz, od = np.concatenate(ozs), np.concatenate(odiff)
    return {"voltage_vectors": len(cases), "currents": int(ab.size), "replicas_fp32": replicas32,
            "replicas_fp64": replicas64, "hops": hops,
            "floor": f"|I| >= {FLOOR:g} x the vector's largest |I| (FP64)",
            "currents_above_floor": int(ab.sum()),
            "count_estimate": _summary(cat["z"], cat["rel"], cat["up"], ab),
            "control_variate_estimate": dict(_summary(catv["z"], catv["rel"], catv["up"], ab),
                                             median_variance_reduction=float(np.median(np.concatenate(vr))),
                                             beta_range=[float(np.concatenate(betas).min()),
                                                         float(np.concatenate(betas).max())],
                                             above_floor=dict(columns=["vector", "electrode", "I_fp64",
                                                                       "rel_diff", "rel_upper3"],
                                                              rows=per_current)),
            "occupancies": int(oz.size), "occupancy_max_abs_z": float(oz.max()),
            "occupancy_frac_within_3sigma": float(np.mean(oz <= 3.0)),
            "occupancy_max_abs_diff": float(od.max()),
            "fp32_inputs": "site energies from the device superposition (kmc_site_energies)",
            "fp32_hops_per_s": len(rows) * hops / t32, "fp64_hops_per_s": len(rows64) * hops / tf64,
            "fp64_s": tf64}


def energy_drift(net, V, dev, n_chains=512, hops=100_000, seed=0):
    """Largest difference (kT) between the engine's incrementally updated
    FP32 energies and their recomputation at the re-anchors (every 1024
    hops), over n_chains chains of the homogeneous workload."""
    from kmc_dn_gb300.engine import Batch, TableSpec, superpose
    spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
    ec, ve = superpose(net.basis, net.comp, V[:n_chains], net.mu, dev=dev)
    b = Batch([spec], np.zeros(n_chains, np.int32), np.full(n_chains, net.kT), None, None,
              np.tile(net.occupation.astype(np.uint8), (n_chains, 1)), np.full(n_chains, hops), seed=seed + 3,
              lanes=16, dev=dev, E_constant_dev=ec, el_energy_dev=ve, measure_drift=True)
    r = b.run().results()
    return {"chains": n_chains, "hops": hops, "reanchor": 1024, "max": float(r["energy_drift"].max()),
            "median": float(np.median(r["energy_drift"]))}


def accuracy_sample(net, V, dev, n_vectors=16, replicas32=512, replicas64=128, hops=300_000, seed=0):
    """``accuracy_of`` on the first ``n_vectors`` voltage vectors of the
    homogeneous workload, and the energy drift its chains see."""
    out = accuracy_of([(net, V[k]) for k in range(n_vectors)], dev, replicas32, replicas64, hops, seed)
    out["energy_drift_kT"] = energy_drift(net, V, dev, seed=seed)
    out["reference"] = ("plain FP64 kernel (bit-exact to the reference loop's hop sequence), "
                        "independent replicas")
    return out


def accuracy_large(dev, seed=0, n_drift=64, drift_hops=100_000, replay_hops=300, n_occ=96, occ_hops=6_000):
    """FP32 error on the large networks (N = 1000, M = 100, 8 electrodes):

    * drift: the largest difference (kT) between the energies the O(N)
      incremental FP32 updates carry and the same energies recomputed from
      scratch, found at the re-anchors (every 1024 hops) of n_drift chains
      over drift_hops hops (the drift the re-anchor bounds; simulation.go:
      107-130 never re-anchors);
    * replay: on a stream whose event uniforms all lie >= 1e-4 of the total
      rate from the FP64 loop's cumulative boundaries, the engine's hop
      sequence against the FP64 oracle's, and along it the largest relative
      error of the FP32 total rate and of the chosen pair's probability;
    * occupations: time-averaged site occupations after occ_hops hops from
      the same start, n_occ independent FP32 chains against n_occ chains of
      the plain FP64 kernel (z-score per site).  Over so few hops an
      N = 1000 network's currents are a handful of electrode events, so
      occupations are the statistic compared."""
    import torch
    from kmc_dn_gb300 import _native, workloads
    from kmc_dn_gb300.engine import Batch, TableSpec, simulate_f64_many
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as orc
    out = {"workload": "N=1000 M=100 networks, 8 electrodes, V~U[-1,1], kT=1, positions mode, 256 lanes"}
    nets = [workloads.large_network(seed=1000 + i) for i in range(max(n_drift, 1))]
    specs = [TableSpec.from_network(n) for n in nets]
    t0 = time.perf_counter()
    b = Batch(specs, np.arange(len(nets)), [n.kT for n in nets], [n.E_constant() for n in nets],
              [n.electrodes[:, 3] for n in nets], [n.occupation.astype(np.uint8) for n in nets], drift_hops,
              seed=seed + 17, pair_mode="positions", lanes=256, measure_drift=True, dev=dev)
    r = b.run().results()
    assert np.all(r["status"] == 0)
    out["energy_drift_kT"] = {"chains": len(nets), "hops": drift_hops, "reanchor": 1024,
                              "max": float(r["energy_drift"].max()), "median": float(np.median(r["energy_drift"])),
                              "s": time.perf_counter() - t0}
    # replay on a boundary-clear stream
    net = nets[0]
    occ = net.occupation.astype(np.uint8)
    t0 = time.perf_counter()
    u, _ = orc.clear_stream(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances, net.E_constant(),
                            net.site_energies(), net.transitions_constant, replay_hops, seed + 5, 1e-4)
    o = orc.numba_replay(net.N, net.P, net.nu, net.kT, net.I_0, net.R, occ, net.distances, net.E_constant(),
                         net.site_energies(), net.transitions_constant, u, record=False)
    rb = Batch([specs[0]], [0], [net.kT], [net.E_constant()], [net.electrodes[:, 3]], [occ], [replay_hops],
               replay=[u], lanes=256, pair_mode="positions", hop_log=True, hop_rates=True, dev=dev)
    rr = rb.run().results()
    hr = rr["hop_rates"][0].astype(np.float64)
    same = int(np.sum(np.all(rr["hop_log"][0] == o["hop_log"], axis=1)))
    out["replay"] = {"hops": replay_hops, "hops_identical": same,
                     "max_rel_err_total_rate": float(np.max(np.abs(hr[:, 0] / o["hop_totals"] - 1))),
                     "max_rel_err_chosen_probability": float(np.max(np.abs(
                         (hr[:, 1] / hr[:, 0]) / (o["hop_rates"] / o["hop_totals"]) - 1))),
                     "s": time.perf_counter() - t0}
    # occupations, FP32 vs FP64 kernel
    t0 = time.perf_counter()
    onet = nets[0]
    ob = Batch([specs[0]], np.zeros(n_occ, np.int32), [onet.kT] * n_occ, [onet.E_constant()] * n_occ,
               [onet.electrodes[:, 3]] * n_occ, [onet.occupation.astype(np.uint8)] * n_occ, occ_hops,
               seed=seed + 29, pair_mode="positions", lanes=256, record=_native.RECORD_NUMBA, dev=dev)
    r32 = ob.run().results()
    assert np.all(r32["status"] == 0)
    ch = dict(N=onet.N, P=onet.P, nu=onet.nu, kT=onet.kT, I_0=onet.I_0, R=onet.R, occupation=onet.occupation,
              distances=onet.distances, E_constant=onet.E_constant(), site_energies=onet.site_energies(),
              transitions_constant=onet.transitions_constant)
    t64, eo64, st64, oit64 = simulate_f64_many([ch] * n_occ, occ_hops, [seed * 31 + 7 + i for i in range(n_occ)],
                                               dev=dev, record=True)
    assert np.all(st64 == 0)
    O32 = np.stack([r32["occ_time"][i] / r32["time"][i] for i in range(n_occ)])
    O64 = np.stack([oit64[i] / t64[i] for i in range(n_occ)])
    osd = np.sqrt(O32.var(0, ddof=1) / n_occ + O64.var(0, ddof=1) / n_occ)
    od = np.abs(O32.mean(0) - O64.mean(0))
    moving = osd > 0
    oz = od[moving] / osd[moving]
    out["occupations"] = {"chains_per_side": n_occ, "hops": occ_hops, "sites": int(od.size),
                          "sites_that_moved": int(moving.sum()),
                          "max_abs_z": float(oz.max()) if oz.size else None,
                          "frac_within_3sigma": float(np.mean(oz <= 3.0)) if oz.size else None,
                          "max_abs_diff": float(od.max()), "s": time.perf_counter() - t0}
    return out


def workload_config(n_chains, hops, world):
    """The workload, the same for both arms of the comparison."""
    return {"workload": WORKLOAD, "n_chains": n_chains, "hops": hops,
            "parallelism": f"independent chains; {world} replica(s), no collective",
            "l2": "flushed between steps (512 MB write)"}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    net, V = build_workload(args.seed, N_CHAINS)
    threads = os.cpu_count() or 1
    n_chains = 256
    from kmc_dn_gb300 import workloads  # noqa: F401
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(net, V, threads, HOPS, n_chains, budget_s=max(2.0, 60.0 / max(1, args.steps + args.warmup)))
        if i >= args.warmup:
            vals.append(r["value"])
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": v, "unit": "hops/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(N_CHAINS, HOPS, world),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "hops/s", "cores": threads, "kind": "port",
                             "sample": r["sample"] + " per step"},
            "e2e": {"value": v, "unit": "hops/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--hops", type=int, default=HOPS)
    ap.add_argument("--chains", type=int, default=N_CHAINS)
    ap.add_argument("--lanes", type=int, default=0)
    # 0: the balanced size (engine.balanced_warps_per_block): 7 warps for the
    # ensemble's 2048 warp items, 293 blocks, at most two per SM (14 warps)
    # on 152 SMs, where 8 warps make 256 blocks, 104 SMs with two (16 warps)
    # and 48 with one (+0.7 % measured for 7)
    ap.add_argument("--warps-per-block", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--persistent", action="store_true",
                    help="uneven workload: persistent launches (resident blocks claim work items)")
    ap.add_argument("--workload", default="homogeneous",
                    choices=["homogeneous", "uneven", "large", "serving", "meanfield"],
                    help="homogeneous: the headline line; the others measure the other "
                         "workloads of the path (one JSON line each)")
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--drain-seconds", type=float, default=120.0)
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    if args.workload != "homogeneous":
        import __graft_entry__
        __graft_entry__.build()
        import torch
        torch.cuda.set_device(local)
        fn = {"uneven": bench_uneven, "large": bench_large, "serving": bench_serving,
              "meanfield": bench_meanfield}[args.workload]
        if rank == 0:
            print(json.dumps(fn(args)), flush=True)
        return

    import torch
    import __graft_entry__
    __graft_entry__.build()
    from kmc_dn_gb300 import _native
    from kmc_dn_gb300.engine import Batch, TableSpec, superpose, simulate_f64

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    from kmc_dn_gb300.parallel import replica_chains, reduce_step
    n_chains, hops = args.chains, args.hops
    chain_offset, stream_ids = replica_chains(rank, n_chains)
    net, V = build_workload(args.seed, n_chains, chain_offset=chain_offset)
    spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
    ec_dev, vel_dev = superpose(net.basis, net.comp, V, net.mu, dev=dev)
    occ0 = np.tile(net.occupation.astype(np.uint8), (n_chains, 1))
    lanes = args.lanes if args.lanes else None
    b = Batch([spec], np.zeros(n_chains, np.int32), np.full(n_chains, net.kT), None, None, occ0,
              np.full(n_chains, hops), streams=stream_ids, seed=args.seed + 1,
              lanes=lanes, warps_per_block=args.warps_per_block or None, dev=dev, E_constant_dev=ec_dev,
              el_energy_dev=vel_dev)
    occ_init = b.occupation.clone()
    stream = torch.cuda.Stream(device=dev)

    def reset():
        b.occupation.copy_(occ_init)
        b.time.zero_()
        b.hops_done.zero_()
        b.electrode_occupation.zero_()
        b.n_pairs.zero_()

    # graph-captured step: state reset + one engine launch per size bin
    with torch.cuda.stream(stream):
        reset()
        b.launch(hops, stream=stream)
    stream.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        reset()
        b.launch(hops, stream=stream)
    launches_per_step = len(b._bins)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # > L2

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            g.replay()
    torch.cuda.synchronize(dev)
    r0 = b.results()
    assert np.all(r0["status"] == 0), "engine reported a chain error"
    pairs_per_step = int(np.sum(r0["n_pairs"]))
    hops_per_step = int(np.sum(r0["hops_done"]))
    assert hops_per_step == n_chains * hops

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    step_ms = []
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)                      # evict L2 between steps (outside the events)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):      # replay and events on one stream
                e0.record(stream)
                g.replay()
                e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - wall0
    clocks = clk.summary()
    total_ms, job_hops = reduce_step(float(np.sum(step_ms)), hops_per_step * args.steps, device=dev)
    value = job_hops / (total_ms * 1e-3)
    ms_per_step = total_ms / args.steps

    # roofline: allowed pairs (one ex2 each) per launch / launch time vs measured ex2 rate
    peak = C.c_double(0)
    _native.check(_native.lib().kmc_measure_ex2_rate(C.byref(peak)))
    achieved = pairs_per_step / (ms_per_step * 1e-3)
    # DRAM bytes of one engine launch, measured by ncu and kept in a
    # machine-readable record beside the profile summary (the kernel's
    # traffic is the one-time state load: it does not grow with hops)
    traffic = None
    tpath = os.path.join(HERE, "profiles", "warp_engine_homogeneous.json")
    if os.path.exists(tpath):
        try:
            traffic = int(json.load(open(tpath))["dram_bytes_per_launch"])
        except (ValueError, KeyError, TypeError):
            traffic = None

    out = None
    if rank == 0:
        # plain single-chain FP64 kernel on the same network (Philox stream)
        f64_hops = 100_000
        se = net.site_energies(V[0])
        simulate_f64(net.N, net.P, net.nu, net.kT, net.I_0, net.R, net.occupation, net.distances,
                     net.E_constant(V[0]), se, net.transitions_constant, 2000, seed=1, dev=dev)
        t0 = time.perf_counter()
        r64 = simulate_f64(net.N, net.P, net.nu, net.kT, net.I_0, net.R, net.occupation, net.distances,
                           net.E_constant(V[0]), se, net.transitions_constant, f64_hops, seed=2, dev=dev)
        f64_rate = f64_hops / (time.perf_counter() - t0)
        assert r64["status"] == 0

        # e2e: the host-buffer C entry point, copies in and out inside the call
        e2e = None
        if not args.no_e2e:
            e2e = run_e2e(net, V, hops, args.seed + 1, lanes or 0)

        acc = acc_large = None
        if not args.no_accuracy:
            acc = accuracy_sample(net, V, dev, seed=args.seed)
            acc_large = accuracy_large(dev, seed=args.seed)

        serving = None
        if not args.no_serving and world == 1:
            serving = serving_sample(seed=args.seed)

        cpu = None
        if not args.no_cpu_baseline and world == 1:
            cpu = cpu_baseline(net, V, os.cpu_count() or 1, hops, min(256, n_chains))

        out = {"metric": METRIC, "value": value, "unit": "hops/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": workload_config(n_chains, hops, world),
               "engine": {"lanes_per_chain": b._bins[0]["G"],
                          "warps_per_block": b._warps(b._bins[0]["G"], b._bins[0]["n_work"]),
                          "launches_per_step": launches_per_step, "graph_captured": True},
               "fp64_single_chain": {"value": f64_rate, "unit": "hops/s", "hops": f64_hops,
                                     "workload": "1 chain, same network, plain FP64 kernel"},
               "ratio_vs_fp64_single_chain": value / world / f64_rate,
               "roofline": {"bound": "sfu", "achieved": achieved / 1e9, "peak": peak.value / 1e9,
                            "unit": "Gexp/s", "frac": achieved / peak.value, "traffic": traffic,
                            "peak_source": "ex2.approx throughput measured live (kmc_measure_ex2_rate)",
                            "work": "allowed pairs A(h) summed over all hops of a launch, one ex2 each"},
               "roofline_hbm": hbm_roofline(traffic, ms_per_step),
               "accuracy_vs_fp64": acc, "accuracy_large_networks": acc_large, "serving": serving,
               "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
               "gpu_launches": launches_per_step * args.steps,
               "wall_s": wall}
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def hbm_roofline(traffic, launch_ms):
    """The same launch against the HBM roofline: its DRAM bytes (ncu) per
    launch time, against the measured copy bandwidth (MEASURED_PEAKS.json, or
    a 6.8 TB/s fallback).  The engine keeps tables and chain state on chip,
    so this fraction is tiny: HBM is not what bounds the hop loop."""
    if traffic is None:
        return None
    peak, src = 6800.0, "fallback 6.8 TB/s (MEASURED_PEAKS.json absent)"
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            peak = float(json.load(open(path))["hbm_gbs"])
            src = "of measured (MEASURED_PEAKS.json hbm_gbs)"
        except (ValueError, KeyError):
            pass
    achieved = traffic / (launch_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_source": src}


def run_e2e(net, V, hops, seed, lanes):
    """Same workload through kmc_run_batch_host: host FP64 inputs copied to
    the device, the run, results copied back, all inside the timed call."""
    from kmc_dn_gb300._native import lib, check
    n = V.shape[0]
    N, P = net.N, net.P
    ec = np.ascontiguousarray(np.concatenate([net.E_constant(v) for v in V]))
    se = np.ascontiguousarray(np.concatenate([np.concatenate([np.zeros(N), v]) for v in V]))
    occ = np.ascontiguousarray(np.tile(net.occupation.astype(np.uint8), n))
    hops_a = np.full(n, hops, np.int64)
    kT = np.full(n, net.kT)
    cg = np.zeros(n, np.int32)
    t_out = np.zeros(n)
    eo = np.zeros(n * P, np.int64)
    st = np.zeros(n, np.int32)
    d = np.ascontiguousarray(net.distances)
    tc = np.ascontiguousarray(net.transitions_constant)
    gN, gP = np.array([N], np.int32), np.array([P], np.int32)
    gnu, gI, gR, goff = np.array([net.nu]), np.array([net.I_0]), np.array([net.R]), np.zeros(1, np.int64)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    L = lib()

    def call():
        occ[:] = np.tile(net.occupation.astype(np.uint8), n)
        check(L.kmc_run_batch_host(1, p(gN), p(gP), p(gnu), p(gI), p(gR), p(goff), p(d), p(tc), n, p(cg),
                                   p(kT), p(ec), p(se), p(occ), p(hops_a), seed, lanes, p(t_out), p(eo), p(st)))
    call()   # warm-up (allocator pools, module load)
    t0 = time.perf_counter()
    reps = 2
    for _ in range(reps):
        call()
    dt = (time.perf_counter() - t0) / reps
    assert np.all(st == 0)
    # bytes kmc_run_batch_host copies each call (its FP32 staging of the
    # energies, the FP64 geometry tables, per-chain parameters and offsets)
    from kmc_dn_gb300.engine import default_lanes
    G = lanes or default_lanes(N + P)
    cpw = max(1, 32 // G)
    n_work = (n + cpw - 1) // cpw
    h2d = (d.nbytes + tc.nbytes + 4 * n * N + 4 * n * P + 4 * n + 4 + 4 + 8 + 4 * n + 8 * n + 8 * n
           + occ.nbytes + hops_a.nbytes + 8 * n + 4 * n_work * cpw)
    d2h = t_out.nbytes + eo.nbytes + occ.nbytes + st.nbytes
    return {"value": n * hops / dt, "unit": "hops/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "api": "kmc_run_batch_host (C ABI, host buffers)"}


def _timed_launch(b, hops, streams, bin_ends=None):
    """One launch per size bin, bin k on streams[k % len(streams)]; the
    time from the first launch to the end of the last.  bin_ends (one
    timing event per bin) receive each bin's end, for per-bin times."""
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for st in streams:
        st.wait_event(e0)
    b.launch(hops, bin_streams=streams)
    for k, st in enumerate(streams):
        ev = bin_ends[k] if bin_ends else torch.cuda.Event()
        ev.record(st)
        torch.cuda.current_stream().wait_event(ev)
    e1.record()
    e1.synchronize()
    if bin_ends:
        for k, ev in enumerate(bin_ends):
            b._bins[k]["seconds"] = e0.elapsed_time(ev) * 1e-3
    return e0.elapsed_time(e1) * 1e-3


def bench_uneven(args):
    """16384 chains, one network each: N ~ U{10..200}, M = 0.1 N, P ~ U{4..12},
    kT log-uniform [0.5, 5], ab/R ~ U[0.5, 2], V ~ U[-2, 2], hops log-uniform
    [1e4, 1e6]; size bins run side by side on their own streams."""
    import torch
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    n = args.chains if args.chains != N_CHAINS else 16384
    t0 = time.perf_counter()
    nets = workloads.uneven_batch(n, seed=args.seed)
    setup_s = time.perf_counter() - t0
    specs = [TableSpec.from_network(net) for net, _ in nets]
    hops = np.array([h for _, h in nets], np.int64)
    lanes, tune_s = None, 0.0
    if not args.no_autotune:
        # lanes per size class picked by timing short runs of each class (autotune.py)
        from kmc_dn_gb300 import autotune
        t0 = time.perf_counter()
        lanes = autotune.choose([s.S for s in specs], pair_mode="positions")
        tune_s = time.perf_counter() - t0
    b = Batch(specs, np.arange(n), [net.kT for net, _ in nets], [net.E_constant() for net, _ in nets],
              [net.electrodes[:, 3] for net, _ in nets], [net.occupation.astype(np.uint8) for net, _ in nets],
              hops, seed=args.seed + 5, pair_mode="positions", lanes=lanes,
              warps_per_block=(getattr(lanes, "warps", None) or 4) if lanes else 4,
              persistent=args.persistent)
    streams = [torch.cuda.Stream() for _ in range(len(b._bins))]
    bin_ends = [torch.cuda.Event(enable_timing=True) for _ in b._bins]
    dt = _timed_launch(b, int(hops.max()), streams, bin_ends)
    r = b.results()
    assert np.all(r["status"] == 0)
    done = int(r["hops_done"].sum())
    S = np.array([s.S for s in specs])
    bins = []
    for bn in b._bins:
        idx = bn["chains"]
        bins.append({"lanes_per_chain": bn["G"], "warps_per_block": b._warps(bn["G"]), "chains": int(len(idx)),
                     "S_range": [int(S[idx].min()), int(S[idx].max())],
                     "hops": int(r["hops_done"][idx].sum()), "max_hops": int(hops[idx].max()),
                     "seconds": bn.get("seconds"),
                     "pairs_per_s": float(r["n_pairs"][idx].sum()) / bn["seconds"] if bn.get("seconds") else None})
    if not args.no_accuracy:
        # FP32 vs FP64 currents per size bin: two networks of each bin, 32
        # replicas each on both kernels (fewer hops for the large bins: the
        # FP64 kernel costs O(S^2) FP64 work per hop)
        for bn, entry in zip(b._bins, bins):
            idx = list(bn["chains"][:2])
            smax = int(S[idx].max())
            ah = 100_000 if smax <= 64 else 30_000 if smax <= 128 else 10_000
            entry["accuracy_vs_fp64"] = accuracy_of([(nets[i][0], nets[i][0].electrodes[:, 3]) for i in idx],
                                                    torch.device("cuda"), replicas32=64, replicas64=32, hops=ah,
                                                    seed=args.seed + 3, pair_mode="positions")
    return {"metric": METRIC, "value": done / dt, "unit": "hops/s", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "uneven batch: 16384 chains, one network each, N~U{10..200}, P~U{4..12}, "
                                   "hops log-uniform [1e4,1e6]", "n_chains": n, "total_hops": done,
                       "pair_mode": "positions", "bins": bins, "host_setup_s": setup_s,
                       "lanes": "autotuned per size class" if lanes else "default by size",
                       "launch": "persistent (work claimed with an atomic counter)" if args.persistent
                                 else "one work item per warp",
                       "autotune_s": tune_s,
                       "autotuned": {str(k): v for k, v in getattr(lanes, "picked", {}).items()}},
            "gpu_launches": len(b._bins), "n_pairs_per_s": float(r["n_pairs"].sum()) / dt}


def bench_large(args):
    """256 chains on their own N=1000, M=100 networks (20x20 density, 8
    electrodes, V ~ U[-1,1]), block groups, positions mode."""
    import torch
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.engine import Batch, TableSpec
    n = 256 if args.chains == N_CHAINS else args.chains
    hops = args.hops if args.hops != HOPS else 100_000
    nets = [workloads.large_network(seed=1000 + i) for i in range(n)]
    specs = [TableSpec.from_network(net) for net in nets]
    lanes, tune_s = args.lanes or 256, 0.0
    if not args.lanes and not args.no_autotune:
        from kmc_dn_gb300 import autotune
        t0 = time.perf_counter()
        lanes = autotune.choose([s.S for s in specs], pair_mode="positions")(specs[0].S)
        tune_s = time.perf_counter() - t0
    b = Batch(specs, np.arange(n), [1.0] * n, [net.E_constant() for net in nets],
              [net.electrodes[:, 3] for net in nets], [net.occupation.astype(np.uint8) for net in nets],
              [10**12] * n, seed=args.seed + 9, pair_mode="positions", lanes=lanes)
    b.launch(1024)
    torch.cuda.synchronize()
    b.n_pairs.zero_()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    b.launch(hops)
    e1.record()
    e1.synchronize()
    dt = e0.elapsed_time(e1) * 1e-3
    r = b.results()
    assert np.all(r["status"] == 0)
    peak = C.c_double(0)
    from kmc_dn_gb300 import _native
    _native.check(_native.lib().kmc_measure_ex2_rate(C.byref(peak)))
    pairs = float(r["n_pairs"].sum())
    return {"metric": METRIC, "value": n * hops / dt, "unit": "hops/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "large networks: 256 chains, own N=1000 M=100 networks, 8 electrodes",
                       "n_chains": n, "hops_per_chain_timed": hops, "lanes_per_chain": lanes,
                       "lanes": "autotuned" if tune_s else "fixed", "autotune_s": tune_s,
                       "pair_mode": "positions"},
            "roofline": {"bound": "sfu", "achieved": pairs / dt / 1e9, "peak": peak.value / 1e9,
                         "unit": "Gexp/s", "frac": pairs / dt / peak.value,
                         "work": "allowed pairs (one ex2 and one rsqrt each in positions mode)"},
            "gpu_launches": 1}


def bench_meanfield(args):
    """Mean-field relaxation (Go probSimulate) of 4096 networks: the N=30,
    P=8 geometry with each network's own voltage vector, 1000 iterations
    each (dn_search's first search stage), FP32 and FP64 rates; the C
    restatement of the Go function on all host threads beside it."""
    import torch
    from concurrent.futures import ThreadPoolExecutor
    from kmc_dn_gb300 import _native
    from kmc_dn_gb300.meanfield import MeanFieldBatch, Network
    n = args.chains if args.chains != N_CHAINS else 4096
    iters = 1000
    net, V = build_workload(args.seed, n)
    nets = [Network(net.N, net.P, net.nu, net.kT, net.I_0, net.R, net.distances, net.transitions_constant,
                    net.E_constant(V[k]), V[k]) for k in range(n)]
    out = {}
    for rates in ("f32", "f64"):
        b = MeanFieldBatch(nets, iters, rates=rates)
        st = torch.cuda.Stream()
        with torch.cuda.stream(st):
            for _ in range(max(1, args.warmup)):
                b.reset()
                b.launch(st)
        st.synchronize()
        ms = []
        for _ in range(args.steps):
            with torch.cuda.stream(st):
                b.reset()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(st)
                b.launch(st)
                e1.record(st)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        r = b.results()
        assert np.all(r["status"] == 0) and np.all(r["iterations"] == iters)
        t = float(np.mean(ms)) * 1e-3
        out[rates] = {"network_iterations_per_s": n * iters / t, "ms_per_launch": t * 1e3,
                      "pairs_per_s": b.pairs_per_iteration * iters / t}
    peak = C.c_double(0)
    _native.check(_native.lib().kmc_measure_ex2_rate(C.byref(peak)))
    # CPU: the oracle's restatement of probSimulate, one network per task
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as orc
    threads = os.cpu_count() or 1

    def cpu_run(k):
        t0 = time.perf_counter()
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda i: orc.prob_simulate(net.N, net.P, net.nu, net.kT, net.I_0, net.R,
                                                    np.full(net.N, 0.5), net.distances, net.E_constant(V[i % n]),
                                                    net.site_energies(V[i % n]), net.transitions_constant, iters),
                        range(k)))
        return time.perf_counter() - t0
    per = cpu_run(threads) / threads                    # calibrate, then about 10 s of CPU work
    k = int(min(n, max(threads, 10.0 / max(per, 1e-6) * threads)))
    cpu_dt = cpu_run(k)
    f32 = out["f32"]
    return {"metric": "mean-field network-iterations/s", "value": f32["network_iterations_per_s"],
            "unit": "network-iterations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": f32["ms_per_launch"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 rates, f64 state", "data": "synthetic",
            "config": {"workload": f"mean-field relaxation: {n} networks (N=30, P=8, own voltages) x {iters} "
                                   "iterations", "n_networks": n, "iterations": iters,
                       "l2": "inputs resident (a few MB), not flushed"},
            "fp64_rates": out["f64"],
            "roofline": {"bound": "sfu", "achieved": f32["pairs_per_s"] / 1e9, "peak": peak.value / 1e9,
                         "unit": "Gexp/s", "frac": f32["pairs_per_s"] / peak.value,
                         "work": "S*S pair rates per network-iteration, one ex2 each"},
            "cpu_baseline": {"value": k * iters / cpu_dt, "unit": "network-iterations/s", "cores": threads,
                             "kind": "port", "sample": f"{k} networks x {iters} iterations, C restatement "
                                                       f"of probSimulate, {cpu_dt:.1f} s wall"},
            "gpu_launches": args.steps}


def _serve_stream(srv, nets, rng, rate, window_s, drain_s, short_first=False, budgets=(10_000, 100_000, 1_000_000)):
    """Submit a Poisson stream (``rate`` per second for ``window_s`` seconds)
    of voltage populations (32..512 vectors, U[-1,1]) on the resident
    geometries with hop budgets from ``budgets``, then wait up to
    ``drain_s`` seconds for them.  With ``short_first`` only the 1e4-hop
    requests are waited for; the rest are cancelled after them.  Returns the
    requests (finished ones carry done_at)."""
    n_req = rng.poisson(rate * window_s)
    arr = np.cumsum(rng.exponential(1.0 / rate, n_req))
    spec = [(int(rng.integers(len(nets))), rng.uniform(-1, 1, (int(rng.integers(32, 513)), 8)),
             int(rng.choice(list(budgets))), int(rng.integers(2**62))) for _ in range(n_req)]
    submitted = []
    t0 = time.perf_counter()
    for (g, V, h, sd), ta in zip(spec, arr):
        delay = t0 + ta - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        submitted.append(srv.submit(g, V, h, sd))
    if short_first:
        t_end = time.perf_counter() + drain_s
        for r in submitted:
            if r.hops == 10_000:
                try:
                    r.future.result(timeout=max(0.0, t_end - time.perf_counter()))
                except Exception:
                    pass
        for r in submitted:
            if r.done_at is None:
                srv.cancel(r)
        srv.wait_idle(timeout=60.0)
    else:
        srv.wait_idle(timeout=drain_s)
    return submitted, time.perf_counter() - t0


def serving_sample(seed=0, rate=200.0, window_s=0.5, sustainable_rate=1.0, sustainable_s=40.0,
                   short_rate=8.0, short_s=12.0, **server_kw):
    """The serving loop on the voltage-search stream: 4 resident geometries
    (N in {30, 60, 120, 240}, M = 0.1 N, 8 electrodes), populations of
    32..512 voltage vectors, hop budgets {1e4, 1e5, 1e6}.

    * isolated: a lone 1e4-hop request per geometry on the idle device;
    * at the specified 200 requests/s (offered work ~140x what the device
      can evaluate, so latency grows with the window): arrivals for
      ``window_s`` s, the 1e4-hop requests waited for, the rest cancelled;
    * at a sustainable rate (~70 % of capacity): arrivals for
      ``sustainable_s`` s, all drained;
    * short requests only (1e4 hops, the voltage search's inner loop) at
      ``short_rate`` per second for ``short_s`` s (about half of what the
      device serves of them), all drained: enough of them per network size
      for a p99 that is more than the largest of a handful.
    p50 / p99 latency (arrival to host result) per hop budget and, for the
    1e4-hop requests, per network size."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.serving import Server, latency_summary
    nets = workloads.serving_geometries(seed=seed)
    srv = Server(nets, quantum=20480, **server_kw)
    rng = np.random.Generator(np.random.PCG64(seed + 77))
    for g in range(len(nets)):          # warm-up: module load, allocator pools
        srv.submit(g, np.zeros((32, 8)), 2048, seed=g)
    srv.run_sync()
    isolated = {}
    for g, net in enumerate(nets):
        for nc in (32, 512):
            r = srv.submit(g, rng.uniform(-1, 1, (nc, 8)), 10_000, seed=1000 + g)
            srv.run_sync()
            isolated[f"N{net.N}_chains{nc}_ms"] = 1e3 * (r.done_at - r.arrival)

    def summary(reqs, wall):
        done = [r for r in reqs if r.done_at is not None and not r.cancelled]
        lat = latency_summary(done)
        short = [r for r in done if r.hops == 10_000]
        for gi, net in enumerate(nets):
            sub = [r for r in short if r.geometry == gi]
            if sub:
                lat[f"hops_10000_N{net.N}"] = latency_summary(sub)["all"]
        return {"requests": len(reqs), "completed": len(done), "wall_s": wall, "latency_ms": lat}

    srv.start()
    srv.hops_done = 0
    reqs, wall = _serve_stream(srv, nets, rng, rate, window_s, drain_s=30.0, short_first=True)
    over = summary(reqs, wall)
    over.update(rate_per_s=rate, arrival_window_s=window_s,
                note="offered load far above capacity: the 1e4-hop requests are served first (strict "
                     "priority), the longer ones are cancelled once those are done")
    srv.hops_done = 0
    reqs, wall = _serve_stream(srv, nets, rng, sustainable_rate, sustainable_s, drain_s=120.0)
    sus = summary(reqs, wall)
    sus.update(rate_per_s=sustainable_rate, arrival_window_s=sustainable_s, hops_per_s=srv.hops_done / wall)
    srv.hops_done = 0
    reqs, wall = _serve_stream(srv, nets, rng, short_rate, short_s, drain_s=60.0, budgets=(10_000,))
    short = summary(reqs, wall)
    short.update(rate_per_s=short_rate, arrival_window_s=short_s, hops_per_s=srv.hops_done / wall)
    srv.stop(drain=False)
    return {"geometries_N": [n.N for n in nets], "isolated_1e4_hops_ms": isolated,
            "at_specified_rate": over, "at_sustainable_rate": sus, "short_requests_at_sustainable_rate": short}


def bench_serving(args):
    """The serving loop alone (``--workload serving``): one stream at
    ``--rate`` for ``--serve-seconds``, drained; p50/p99 per budget."""
    from kmc_dn_gb300 import workloads
    from kmc_dn_gb300.serving import Server, latency_summary
    nets = workloads.serving_geometries(seed=args.seed)
    srv = Server(nets, quantum=20480)
    rng = np.random.Generator(np.random.PCG64(args.seed + 77))
    for g in range(4):
        srv.submit(g, np.zeros((32, 8)), 2048, seed=g)
    srv.run_sync()
    srv.hops_done = 0
    srv.start()
    reqs, wall = _serve_stream(srv, nets, rng, args.rate, args.serve_seconds, drain_s=args.drain_seconds)
    srv.stop(drain=False)
    done = [r for r in reqs if r.done_at is not None]
    lat = latency_summary(done)
    for gi, net in enumerate(nets):
        sub = [r for r in done if r.geometry == gi]
        if sub:
            lat[f"N{net.N}"] = latency_summary(sub)
    return {"metric": METRIC, "value": srv.hops_done / wall, "unit": "hops/s", "n_gpus": 1, "steps": 1,
            "warmup": 1, "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "serving: Poisson voltage-search requests on 4 resident geometries",
                       "rate_per_s": args.rate, "arrival_window_s": args.serve_seconds,
                       "requests": len(reqs), "completed": len(done),
                       "quantum_hops": srv.quantum, "quantum_long_hops": srv.quantum_long,
                       "long_thread_budget": srv.long_thread_budget},
            "latency": lat, "gpu_launches": srv.launches}


if __name__ == "__main__":
    main()
