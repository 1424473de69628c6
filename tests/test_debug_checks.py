"""The debug-checks build (python -m kmc_dn_gb300.build --debug-checks,
-DKMC_DEBUG_CHECKS): the hop loop checks its decoded pair, chosen event, hop
sites and list-rebuild indices every hop and stops a chain with
KMC_ERR_INVALID instead of using a bad index (compute-sanitizer is not
available).  Mixed sizes, lane counts, both pair modes, record and replay
run clean under it, with results bit-identical to the release build."""
import json
import os
import subprocess
import sys

import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, %(repo)r)
from kmc_dn_gb300 import _native, workloads
from kmc_dn_gb300.engine import Batch, TableSpec
from kmc_dn_gb300.rng import replay_uniforms
out = {"lib": _native.LIB_PATH}
nets = [n for n, _ in workloads.uneven_batch(48, seed=5, hops_range=(3000, 3000))]
specs = [TableSpec.from_network(n) for n in nets]
for mode in ("table", "positions"):
    for lanes in (None, 8, 32, 128, 512):
        b = Batch(specs, np.arange(len(nets)), [n.kT for n in nets], [n.E_constant() for n in nets],
                  [n.electrodes[:, 3] for n in nets], [n.occupation.astype(np.uint8) for n in nets], 3000,
                  seed=11, lanes=lanes, pair_mode=mode, record=_native.RECORD_GO)
        r = b.run().results()
        out[f"{mode}/{lanes}"] = dict(status=r["status"].tolist(), hops=r["hops_done"].tolist(),
                                      time=r["time"].tolist(),
                                      eo=[x.tolist() for x in r["electrode_occupation"]])
net = workloads.plain_network(0)
u = replay_uniforms(7, 2 * 2000)
spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
r = Batch([spec], [0], [net.kT], [net.E_constant()], [net.electrodes[:, 3]], [net.occupation.astype(np.uint8)],
          [2000], replay=[u], lanes=8).run().results()
out["replay"] = dict(status=r["status"].tolist(), time=r["time"].tolist(), eo=r["electrode_occupation"][0].tolist())
print(json.dumps(out))
"""


def _run(lib):
    env = dict(os.environ)
    env["KMC_DN_GB300_LIB"] = lib
    p = subprocess.run([sys.executable, "-c", SCRIPT % {"repo": REPO}], env=env, capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return json.loads(p.stdout.strip().splitlines()[-1])


def test_debug_checks_build_runs_clean_and_matches_release(engine_lib):
    from kmc_dn_gb300 import build
    dbg = build.build(debug_checks=True)
    a = _run(dbg)
    b = _run(build.LIB)
    assert a["lib"] == dbg and b["lib"] == build.LIB
    for k, v in a.items():
        if k == "lib":
            continue
        assert all(s == 0 for s in v["status"]), (k, v["status"])
        assert v == b[k], k


CROSS = r"""
import json, sys
import numpy as np
sys.path.insert(0, %(repo)r)
from kmc_dn_gb300 import _native, workloads
from kmc_dn_gb300.engine import Batch, TableSpec
out = {"lib": _native.LIB_PATH, "hops": 0, "mismatch": 0, "status": 0}
net, V = workloads.homogeneous_ensemble(4096, 0)
spec = TableSpec(net.N, net.P, net.nu, net.I_0, net.R, net.distances, net.transitions_constant)
b = Batch([spec], np.zeros(4096, np.int32), np.full(4096, net.kT), [net.E_constant(v) for v in V], list(V),
          np.tile(net.occupation.astype(np.uint8), (4096, 1)), np.full(4096, 3072), seed=3, lanes=16,
          count_select_mismatch=True)
r = b.run().results()
out["hops"] += int(r["hops_done"].sum()); out["mismatch"] += int(r["select_mismatch"].sum())
out["status"] += int(np.abs(r["status"]).sum())
nets = [workloads.large_network(seed=s, N=300, M=30) for s in range(8)]
specs = [TableSpec.from_network(n) for n in nets]
for lanes in (32, 128, 512):
    b = Batch(specs, np.arange(8), [1.0] * 8, [n.E_constant() for n in nets], [n.electrodes[:, 3] for n in nets],
              [n.occupation.astype(np.uint8) for n in nets], 20000, seed=4, lanes=lanes, pair_mode="positions",
              count_select_mismatch=True)
    r = b.run().results()
    out["hops"] += int(r["hops_done"].sum()); out["mismatch"] += int(r["select_mismatch"].sum())
    out["status"] += int(np.abs(r["status"]).sum())
print(json.dumps(out))
"""


def test_fp64_cross_check_of_the_selection_finds_no_difference(engine_lib):
    """In the debug-checks build every hop also selects its event with an FP64
    scan and compare over the same FP32 per-thread sums (the precision the
    reference's final cumulative compare has, kmc_dopant_networks.py:91-110)
    and counts the hops where that picks another pair than the engine's exact
    integer compare: over 1.3*10^7 hops (warp slices on the N = 30 network,
    warp and block groups on N = 300 networks) the count is zero."""
    from kmc_dn_gb300 import build
    dbg = build.build(debug_checks=True)
    env = dict(os.environ)
    env["KMC_DN_GB300_LIB"] = dbg
    p = subprocess.run([sys.executable, "-c", CROSS % {"repo": REPO}], env=env, capture_output=True, text=True,
                       timeout=900)
    assert p.returncode == 0, p.stderr[-2000:]
    out = json.loads(p.stdout.strip().splitlines()[-1])
    assert out["lib"] == dbg and out["status"] == 0
    assert out["hops"] >= 10**7
    assert out["mismatch"] == 0, out
