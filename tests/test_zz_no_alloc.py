"""kmc_simulate_f64_static: the FP64 hop loop for callers that cannot
allocate device memory when they call it (a host that owns the device through
its own memory pool, or a latency-bound loop that cannot afford
cudaMalloc/cudaFree).  Its workspace is a fixed array inside the library; the
results must equal those of kmc_simulate_f64 with a caller workspace, call
after call, whatever an earlier call left in that array.

This file is collected last on purpose; it needs nothing from other tests.
"""
import ctypes as C

import numpy as np
import pytest

from kmc_dn_gb300.rng import replay_uniforms

pytestmark = pytest.mark.gpu


def _call(entry, net, hops, *, uniforms=None, seed=0, record=True):
    """Run one chain through `entry` ("workspace" or "static") via the C ABI
    with fresh device buffers; return host copies of every output."""
    import torch
    from kmc_dn_gb300 import _native
    L = _native.lib()
    d = torch.device("cuda")
    N, P = net["N"], net["P"]
    S = N + P
    f64 = torch.float64
    t = lambda a, dt=f64: torch.as_tensor(np.ascontiguousarray(a)).to(dtype=dt, device=d)  # noqa: E731
    occ = t(net["occupation"], torch.uint8)
    dist, tc = t(net["distances"]), t(net["transitions_constant"])
    ec, se = t(net["E_constant"]), t(net["site_energies"])
    eo = torch.zeros(max(P, 1), dtype=torch.int64, device=d)
    traffic = torch.zeros(S * S, dtype=f64, device=d)
    oit = torch.zeros(max(N, 1), dtype=f64, device=d)
    u = t(uniforms) if uniforms is not None else None
    log = torch.zeros(2 * hops, dtype=torch.int32, device=d)
    t_out = torch.zeros(1, dtype=f64, device=d)
    st = torch.zeros(1, dtype=torch.int32, device=d)
    p = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None  # noqa: E731
    common = [N, P, float(net["nu"]), float(net["kT"]), float(net["I_0"]), float(net["R"]), p(occ), p(dist),
              p(ec), p(se), p(tc), p(eo), hops, int(record), p(traffic), p(oit), p(u), seed, p(log),
              p(t_out), p(st)]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if entry == "workspace":
        wsb = L.kmc_simulate_f64_workspace_size(S)
        ws = torch.empty(wsb, dtype=torch.uint8, device=d)
        rc = L.kmc_simulate_f64(*common, p(ws), wsb, stream)
    else:
        rc = L.kmc_simulate_f64_static(*common, stream)
    _native.check(rc)
    torch.cuda.synchronize()
    return dict(occupation=occ.cpu().numpy(), eo=eo.cpu().numpy()[:P], traffic=traffic.cpu().numpy(),
                oit=oit.cpu().numpy()[:N], log=log.cpu().numpy(), time=float(t_out.item()),
                status=int(st.item()))


def _network(seed, N):
    from kmc_dn_gb300 import workloads
    L = float(np.sqrt(N / workloads.DENSITY))
    rng = np.random.Generator(np.random.PCG64(seed))
    net = workloads.make_network(rng, N, max(1, N // 10), L, L, workloads.edge_thirds(L),
                                 voltages=rng.uniform(-1, 1, 8), I_0=50.0, cells=60)
    return dict(N=net.N, P=net.P, nu=net.nu, kT=net.kT, I_0=net.I_0, R=net.R,
                occupation=net.occupation.astype(np.uint8), distances=net.distances,
                transitions_constant=net.transitions_constant, E_constant=net.E_constant(),
                site_energies=net.site_energies())


def _same(a, b):
    assert a["status"] == b["status"] == 0
    np.testing.assert_array_equal(a["log"], b["log"])
    np.testing.assert_array_equal(a["occupation"], b["occupation"])
    np.testing.assert_array_equal(a["eo"], b["eo"])
    np.testing.assert_array_equal(a["traffic"], b["traffic"])
    assert abs(a["time"] - b["time"]) <= 1e-12 * abs(b["time"])
    np.testing.assert_allclose(a["oit"], b["oit"], rtol=1e-12, atol=0)


def test_static_workspace_matches_caller_workspace_twice(engine_lib):
    # first call: the larger network (more of the array in use), replay stream
    big = _network(11, 90)
    u = replay_uniforms(5, 2 * 3000)
    _same(_call("static", big, 3000, uniforms=u), _call("workspace", big, 3000, uniforms=u))
    # second call right after, on a smaller network with the generator: the
    # first call's leftovers in the shared array must not leak into it
    small = _network(12, 30)
    _same(_call("static", small, 4000, seed=9, record=False),
          _call("workspace", small, 4000, seed=9, record=False))


def test_static_workspace_rejects_networks_beyond_its_size(engine_lib):
    from kmc_dn_gb300 import _native
    L = _native.lib()
    rc = L.kmc_simulate_f64_static(200, 8, 1.0, 1.0, 1.0, 1.0, *([None] * 6), 10, 0, None, None, None,
                                   0, None, None, None, None)
    assert rc == _native.KMC_ERR_INVALID
    code, msg = _native.last_error()
    assert "at most 128" in msg
