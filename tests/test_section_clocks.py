"""The section-clocks build (python -m kmc_dn_gb300.build --section-clocks,
-DKMC_SECTION_CLOCKS) times the phases of the FP32 hop loop; its per-phase
cycles per hop add up to about the launch's wall time per hop."""
import json
import subprocess
import sys

import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu


def test_section_clocks_cover_the_hop(engine_lib):
    p = subprocess.run([sys.executable, "-m", "kmc_dn_gb300.section_clocks", "--hops", "20000"], cwd=REPO,
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    r = json.loads(p.stdout.strip().splitlines()[-1])
    assert r["library"] == "libkmc_dn_gb300_clocks.so"
    cyc = r["cycles_per_hop"]
    assert set(cyc) == {"top", "pairs", "uniforms", "scan", "search", "clock", "rebuild", "update"}
    assert all(v > 0 for v in cyc.values())
    assert max(cyc, key=cyc.get) == "pairs"
    # thread 0's phases span its whole hop: at 1-2.1 GHz the sum is the wall time per hop
    wall_cycles_lo, wall_cycles_hi = r["wall_us_per_hop"] * 1.0e3, r["wall_us_per_hop"] * 2.1e3
    assert 0.7 * wall_cycles_lo <= r["sum_cycles_per_hop"] <= 1.05 * wall_cycles_hi
