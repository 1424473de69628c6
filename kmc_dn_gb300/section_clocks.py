"""Where a hop's time goes: per-phase SM-clock cycles of the FP32 engine.

    python -m kmc_dn_gb300.section_clocks [--workload homogeneous|large] [--hops H]

builds the section-clocks library (``build.py --section-clocks``: the same
engine compiled with -DKMC_SECTION_CLOCKS), runs one launch of the workload
through it in a child process and prints one JSON line: for each phase of
the hop loop, the cycles per hop seen by thread 0 of a group (its warp's
time, including the issue slots other warps took) and its share.  The
phases are those of the hop loop in csrc/kmc_f32_engine.cuh:

  top       the cancel / time-budget / re-anchor checks at the top of a hop
  pairs     the rate walk over the thread's run of allowed pairs
  uniforms  the clock and event uniforms (Philox refill, broadcast)
  scan      the double-float group scan, the target and the event thread
  search    the search in that thread's run, the event's (from, to)
  clock     the clock advance
  rebuild   the O(N) energy update and the source/target list rebuild
  update    occupancy bits, electrode counters, record, hop count

The timer reads cost a few percent of the hop; the wall cycles per hop of
the same launch are printed beside the sum for comparison.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys

PHASES = ("top", "pairs", "uniforms", "scan", "search", "clock", "rebuild", "update")


def _measure(workload, hops):
    import ctypes as C

    import numpy as np
    import torch

    from . import _native, workloads
    from .engine import Batch, TableSpec

    if workload == "homogeneous":
        n = 4096
        net, V = workloads.homogeneous_ensemble(n, 0)
        spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
        b = Batch([spec], np.zeros(n, np.int32), np.full(n, net.kT), [net.E_constant(v) for v in V], list(V),
                  np.tile(net.occupation.astype(np.uint8), (n, 1)), np.full(n, hops), seed=1, lanes=16,
                  warps_per_block=None)
        desc = "4096 chains, N=30 M=3 P=8, 16 lanes per chain, table mode"
    else:
        n = 256
        nets = [workloads.large_network(seed=1000 + i) for i in range(n)]
        specs = [TableSpec.from_network(x) for x in nets]
        b = Batch(specs, np.arange(n), [1.0] * n, [x.E_constant() for x in nets],
                  [x.electrodes[:, 3] for x in nets], [x.occupation.astype(np.uint8) for x in nets],
                  [10**12] * n, seed=9, pair_mode="positions", lanes=512)
        desc = "256 chains, own N=1000 M=100 networks, 512 lanes per chain, positions mode"
    L = _native.lib()
    out = (C.c_uint64 * (len(PHASES) + 1))()
    b.launch(min(hops, 1024))                       # warm-up launch
    torch.cuda.synchronize()
    _native.check(L.kmc_section_clocks(out, 1))     # zero the counters
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.launch(hops)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    _native.check(L.kmc_section_clocks(out, 1))
    r = b.results()
    if not np.all(r["status"] == 0):
        raise RuntimeError("a chain stopped with an error")
    n_hops = int(out[len(PHASES)])
    per_hop = {k: out[i] / n_hops for i, k in enumerate(PHASES)}
    total = sum(per_hop.values())
    return {"workload": workload, "config": desc, "hops_per_chain": hops, "library": os.path.basename(_native.LIB_PATH),
            "cycles_per_hop": {k: round(v, 1) for k, v in per_hop.items()},
            "share": {k: round(v / total, 4) for k, v in per_hop.items()},
            "sum_cycles_per_hop": round(total, 1), "launch_ms": ms,
            "wall_us_per_hop": ms * 1e3 / hops}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", choices=("homogeneous", "large"), default="homogeneous")
    ap.add_argument("--hops", type=int, default=0, help="hops per chain (default 100000 / 2000)")
    ap.add_argument("--child", action="store_true", help=argparse.SUPPRESS)
    a = ap.parse_args(argv)
    hops = a.hops or (100_000 if a.workload == "homogeneous" else 2000)
    if a.child:
        print(json.dumps(_measure(a.workload, hops)), flush=True)
        return 0
    from . import build
    lib = build.build(section_clocks=True)
    env = dict(os.environ, KMC_DN_GB300_LIB=lib)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = [sys.executable, "-m", "kmc_dn_gb300.section_clocks", "--workload", a.workload, "--hops", str(hops),
           "--child"]
    return subprocess.call(cmd, env=env, cwd=root)


if __name__ == "__main__":
    sys.exit(main())
