"""Generate the golden vectors under tests/golden/ from the reference itself.

Runs the reference's own hop loop, ``_simulate_discrete_record``
(kmc_dopant_networks.py:33-135), as plain Python: ``numba`` is replaced by a
stub whose ``jit`` is the identity and ``fenics`` by an empty module (only
the ``kmc_dn`` class needs it, and it is not used here).  The module-global
``np`` seen by the hop loop is swapped for a shim whose ``random`` draws from
a replay stream (``kmc_dn_gb300.rng.replay_uniforms``):
``np.random.exponential(scale)`` returns ``-log(1 - u) * scale`` and
``np.random.rand()`` returns the next u, so each hop consumes exactly two
uniforms, clock first, then event.

The hop loop is called one hop at a time so that every hop's (from, to) pair
can be read off the change of ``occupation`` / ``electrode_occupation``; this
is the same computation as one long call because the loop recomputes every
site energy and rate from the occupation on each hop, and the caller
accumulates time and the record arrays in the loop's own order.

It also copies the set-up data of a sample of the reference's statistical
fixtures (thesis_indrek/tests/*/test*.kmc, read with a restricted unpickler)
into small .npz files.

Usage (needs the reference checkout; the outputs are committed):
    python tests/golden/make_golden.py [--reference /path/to/kmc_dn] [--quick]
"""
from __future__ import annotations

import argparse
import glob
import os
import pickle
import sys
import time
import types
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from kmc_dn_gb300.rng import replay_uniforms  # noqa: E402
from kmc_dn_gb300 import workloads, geometry as geo  # noqa: E402

_REF = None


def load_reference(path):
    """Import kmc_dopant_networks from the reference checkout with stubs."""
    global _REF
    if _REF is not None:
        return _REF
    numba = types.ModuleType("numba")

    def jit(*a, **k):
        if len(a) == 1 and callable(a[0]) and not k:
            return a[0]
        return lambda f: f
    numba.jit = jit
    sys.modules.setdefault("numba", numba)
    sys.modules.setdefault("fenics", types.ModuleType("fenics"))
    sys.path.insert(0, path)
    cwd = os.getcwd()
    os.chdir(path)
    try:
        import kmc_dopant_networks as ref
    finally:
        os.chdir(cwd)
    _REF = ref
    return ref


class _Stream:
    def __init__(self, u):
        self.u = u
        self.k = 0

    def exponential(self, scale=1.0):
        u = self.u[self.k]
        self.k += 1
        return -np.log(1 - u) * scale

    def rand(self):
        u = self.u[self.k]
        self.k += 1
        return u


class _NpShim:
    def __init__(self, stream):
        self.random = stream

    def __getattr__(self, name):
        return getattr(np, name)


class _FixtureUnpickler(pickle.Unpickler):
    """Only the numpy reconstruction globals the .kmc files use."""
    ALLOWED = {("numpy.core.multiarray", "_reconstruct"), ("numpy", "ndarray"),
               ("numpy", "dtype"), ("numpy.core.multiarray", "scalar"),
               ("numpy._core.multiarray", "_reconstruct"), ("numpy._core.multiarray", "scalar")}

    def find_class(self, module, name):
        if (module, name) not in self.ALLOWED:
            raise pickle.UnpicklingError(f"global {module}.{name} not allowed")
        import importlib
        return getattr(importlib.import_module(module), name)


def read_fixture(path):
    with open(path, "rb") as f:
        return _FixtureUnpickler(f).load()


def run_reference(ref_path, case):
    """Replay one case through the reference hop loop; returns a dict."""
    ref = load_reference(ref_path)
    N, P = case["N"], case["P"]
    S = N + P
    hops = case["hops"]
    u = replay_uniforms(case["seed"], 2 * hops)
    shim = _NpShim(_Stream(u))
    ref.np = shim
    occ = case["occupation"].astype(bool).copy()
    eo = np.zeros(P, dtype=np.int64)
    se = case["site_energies"].astype(np.float64).copy()
    trans = np.zeros((S, S))
    problist = np.zeros(S * S)
    total_time = 0.0
    traffic = np.zeros((S, S))
    oit = np.zeros(N)
    log = np.zeros((hops, 2), dtype=np.int16)
    ckpt_every = case.get("ckpt", 1000)
    times = []
    t0 = time.time()
    for h in range(hops):
        occ_before = occ.copy()
        eo_before = eo.copy()
        t, occ, eo, tr, oi = ref._simulate_discrete_record(
            N, P, case["nu"], case["kT"], case["I_0"], case["R"], 0, occ,
            case["distances"], case["E_constant"], se, case["transitions_constant"],
            trans, problist, eo, 1, record=True)
        total_time += t
        traffic += tr
        oit += oi
        src = np.flatnonzero(occ_before & ~occ)
        dst = np.flatnonzero(~occ_before & occ)
        esrc = np.flatnonzero(eo < eo_before)
        edst = np.flatnonzero(eo > eo_before)
        fr = int(src[0]) if len(src) else N + int(esrc[0])
        to = int(dst[0]) if len(dst) else N + int(edst[0])
        log[h] = (fr, to)
        if (h + 1) % ckpt_every == 0:
            times.append(total_time)
    ref.np = np
    assert shim.random.k == 2 * hops
    out = dict(case)
    out.update(hop_log=log, time=total_time, time_ckpt=np.array(times),
               final_occupation=occ.astype(np.uint8), final_electrode_occupation=eo,
               traffic=traffic, occupations_in_time=oit, wall_s=time.time() - t0)
    return out


def fixture_case(ref_path, rel, seed, hops):
    d = read_fixture(os.path.join(ref_path, rel))
    N, P = int(d["N"]), int(d["P"])
    se = np.zeros(N + P)
    se[N:] = d["electrodes"][:, 3]
    return dict(name="fixture_" + "_".join(rel.split("/")[-2:]).replace(".kmc", ""), N=N, P=P,
                nu=float(d["nu"]), kT=float(d["kT"]), I_0=float(d["I_0"]), R=float(d["R"]),
                distances=d["distances"], transitions_constant=d["transitions_constant"],
                E_constant=d["E_constant"], site_energies=se,
                occupation=d["occupation"].astype(np.uint8), seed=seed, hops=hops)


def network_case(name, net, seed, hops, occupation=None):
    occ = net.occupation if occupation is None else occupation
    return dict(name=name, N=net.N, P=net.P, nu=net.nu, kT=net.kT, I_0=net.I_0, R=net.R,
                distances=net.distances, transitions_constant=net.transitions_constant,
                E_constant=net.E_constant(), site_energies=net.site_energies(),
                occupation=np.asarray(occ).astype(np.uint8), seed=seed, hops=hops)


def small_cases(hops):
    cases = []
    rng = np.random.Generator(np.random.PCG64(7))
    # closed system (no electrodes): constant hole number
    acc, _ = geo.place_dopants(rng, 8, 0, 1.0, 1.0, 0.0)
    R, _ = geo.dimensionless_R(8, 1.0, 1.0, 0.0)
    dist = geo.site_distances(acc, np.zeros((0, 4)))
    occ = np.zeros(8, np.uint8); occ[:4] = 1
    cases.append(dict(name="closed_N8_P0", N=8, P=0, nu=1.0, kT=1.0, I_0=1.0, R=R,
                      distances=dist, transitions_constant=geo.transitions_constant(dist, 1.0, R),
                      E_constant=rng.uniform(-1, 1, 8), site_energies=np.zeros(8),
                      occupation=occ, seed=101, hops=hops))
    # single acceptor between two electrodes (validation/set/set.py:40-60 layout)
    acc1 = np.array([[0.5, 0.0, 0.0]])
    el = np.array([[0.0, 0, 0, 1.0], [1.0, 0, 0, 0.0]])
    d1 = geo.site_distances(acc1, el)
    cases.append(dict(name="set_N1_P2", N=1, P=2, nu=1.0, kT=1.0, I_0=1.0, R=1.0,
                      distances=d1, transitions_constant=geo.transitions_constant(d1, 1.0, 1e5),
                      E_constant=np.array([0.5]), site_energies=np.array([0.0, 1.0, 0.0]),
                      occupation=np.zeros(1, np.uint8), seed=102, hops=hops))
    # starts with every acceptor full / empty, and a mid-size network
    for name, seed, N, fill in (("full_N10_P3", 103, 10, 1), ("empty_N10_P3", 104, 10, 0)):
        r = np.random.Generator(np.random.PCG64(seed))
        L = float(np.sqrt(N / workloads.DENSITY))
        net = workloads.make_network(r, N, 1, L, L, workloads.perimeter_electrodes(L, 3),
                                     voltages=r.uniform(-2, 2, 3), I_0=50.0, cells=40)
        cases.append(network_case(name, net, seed, hops, np.full(N, fill, np.uint8)))
    r = np.random.Generator(np.random.PCG64(105))
    L = float(np.sqrt(60 / workloads.DENSITY))
    net = workloads.make_network(r, 60, 6, L, L, workloads.edge_thirds(L),
                                 voltages=r.uniform(-1, 1, 8), I_0=50.0, kT=0.7, cells=60)
    cases.append(network_case("mid_N60_P8", net, 105, hops))
    return cases


def time_reference(ref_path, hops):
    """Wall time of one call of the reference's _simulate_discrete_record
    (kmc_dopant_networks.py:33-135, numba stubbed out, numpy's own random
    generator) for `hops` hops on the benchmark network."""
    ref = load_reference(ref_path)
    net = workloads.plain_network(0)
    S = net.S
    np.random.seed(1)
    t0 = time.perf_counter()
    ref._simulate_discrete_record(net.N, net.P, net.nu, net.kT, net.I_0, net.R, 0,
                                  net.occupation.astype(bool).copy(), net.distances, net.E_constant(),
                                  net.site_energies(), net.transitions_constant, np.zeros((S, S)),
                                  np.zeros(S * S), np.zeros(net.P, dtype=np.int64), hops, record=False)
    dt = time.perf_counter() - t0
    print(f"reference _simulate_discrete_record (plain Python, 1 core): {hops} hops in {dt:.1f} s "
          f"= {hops / dt:.1f} hops/s")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("KMC_DN_REFERENCE", "/root/reference"))
    ap.add_argument("--quick", action="store_true", help="short runs only")
    ap.add_argument("--long-hops", type=int, default=100_000)
    ap.add_argument("--only", default=None)
    ap.add_argument("--time-reference", type=int, default=0, metavar="HOPS",
                    help="only time the reference's own hop loop (plain Python, one core) for "
                         "HOPS hops on the N=30, P=8 benchmark network and print hops/s")
    args = ap.parse_args()
    ref = args.reference
    if args.time_reference:
        return time_reference(ref, args.time_reference)
    long_hops = 2000 if args.quick else args.long_hops

    cases = [fixture_case(ref, "thesis_indrek/tests/rnd_min_max/test0.kmc", 11, long_hops),
             network_case("plain_N30_P8", workloads.plain_network(0), 12, long_hops)]
    cases += small_cases(3000)
    if args.only:
        cases = [c for c in cases if args.only in c["name"]]
    with ProcessPoolExecutor(max_workers=min(8, len(cases))) as ex:
        futs = [ex.submit(run_reference, ref, c) for c in cases]
        for f in futs:
            out = f.result()
            name = out.pop("name")
            np.savez_compressed(os.path.join(HERE, f"replay_{name}.npz"), **out)
            print(f"{name}: {out['hops']} hops in {out['wall_s']:.1f}s, time={out['time']!r}")

    # set-up data of a sample of the reference's statistical fixtures
    keys = ["N", "M", "P", "R", "ab", "I_0", "kT", "nu", "xdim", "ydim", "zdim", "res", "mu",
            "acceptors", "donors", "electrodes", "distances", "transitions_constant",
            "E_constant", "eV_constant", "comp_constant", "mean_currents", "stddev_currents",
            "occupation", "time", "electrode_occupation"]
    for sub in ("rnd_min_max", "rnd_min_max5M", "XOR_wide", "XOR_wide5M"):
        files = sorted(glob.glob(os.path.join(ref, "thesis_indrek/tests", sub, "test*.kmc")),
                       key=lambda p: int(os.path.basename(p)[4:-4]))[:12]
        recs = [read_fixture(p) for p in files]
        arrs = {k: np.array([np.asarray(r[k], dtype=np.float64) for r in recs]) for k in keys}
        arrs["files"] = np.array([os.path.relpath(p, ref) for p in files])
        np.savez_compressed(os.path.join(HERE, f"fixtures_{sub}.npz"), **arrs)
        print(f"fixtures_{sub}: {len(recs)}")


if __name__ == "__main__":
    main()
