"""Serving loop: continuous batching over resident interpolants.

Every request's result in the mix (merged persistent launches, overlapping
streams, staggered arrivals, tight memory budget) must equal its result alone
(same kernels per 128-point tile: bit-identical, tolerance 0).
"""
import numpy as np
import pytest
import torch

import functions as fns

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fleet():
    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes

    specs = [("a", "leja", 6, 6.0, 1), ("b", "gh", 9, 6.0, 4), ("c", "leja", 40, 6.5, 1), ("d", "leja", 12, 6.0, 20),
             ("e", "gh", 30, 5.5, 2)]
    ips = {}
    for name, kind, d, t, d_out in specs:
        k = np.log((2 + np.arange(d)) / np.log(2))
        gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
        f = fns.rational_vec(d, d_out, seed=d) if kind == "leja" else fns.exponential(d, d_out, seed=d)
        ips[name] = SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=t, d_out=d_out, f=f)
    return ips


def _requests(ips, seed, n=40):
    from smolyax_gb300.serving import Request

    rng = np.random.default_rng(seed)
    names = sorted(ips)
    reqs = []
    for i in range(n):
        name = names[rng.integers(len(names))]
        ip = ips[name]
        P = int(np.exp(rng.uniform(0, np.log(3000))))
        x = rng.uniform(-0.9, 0.9, (P, ip.d_in))
        op = "grad" if rng.random() < 0.2 else "eval"
        prec = "fp64" if (op == "eval" and rng.random() < 0.2) else "fp32"
        reqs.append(Request(name, x, op=op, precision=prec))
    return reqs


def _alone(ips, req):
    x = torch.as_tensor(req.x, device="cuda")
    ip = ips[req.name]
    if req.op == "eval":
        return ip(x, precision=req.precision).cpu().numpy()
    g = torch.ones(req.points, ip.d_out, dtype=torch.float32, device="cuda")
    return ip.spectral_plan().vjp(x, g, need_x=True, need_coef=False)[0].cpu().numpy()


def test_mix_equals_alone(fleet):
    from smolyax_gb300.serving import Server, replay

    reqs = _requests(fleet, 11)
    server = Server(fleet, memory_budget=0.25, n_streams=4)
    # a burst of 12 requests at t = 0 (merged launches), then staggered arrivals
    arrivals = np.concatenate([np.zeros(12), np.random.default_rng(3).exponential(0.002, len(reqs) - 12).cumsum()])
    wall = replay(server, arrivals, reqs)
    st = server.stats()
    print("served %d requests in %.3fs, %d launches (%d merged), p50 %.2f ms p99 %.2f ms" % (
        st["completed"], wall, st["launches"], st["batch_launches"], st["p50_ms"], st["p99_ms"]))
    assert st["completed"] == len(reqs) and st["rejected"] == 0
    assert st["batch_launches"] >= 1 and st["launches"] < len(reqs)
    for r in reqs:
        assert r.error is None
        np.testing.assert_array_equal(r.result, _alone(fleet, r))


def test_burst_and_rejection(fleet):
    from smolyax_gb300.serving import Request, Server

    reqs = _requests(fleet, 12, n=25)
    server = Server(fleet, memory_budget=1.0, n_streams=8)
    for r in reqs:
        server.submit(r)
    big = server.submit(Request("c", np.zeros((4_000_000, fleet["c"].d_in)), op="eval"))
    server.drain()
    assert big.error is not None and big.result is None
    for r in reqs:
        np.testing.assert_array_equal(r.result, _alone(fleet, r))


def test_merged_gradients_tensor_core_and_fp64_equal_alone(fleet):
    """A burst of gradient requests and tensor-core evaluations of one
    interpolant and FP64 evaluations of another, submitted together: each
    group is served by one merged call (one launch per interpolant, operation
    and precision), and every request's rows equal its result alone.  The
    pinned staging arena is made too small for some inputs (one-off pinned
    buffers are then used)."""
    from smolyax_gb300.serving import Request, Server

    rng = np.random.default_rng(21)
    reqs = []
    for P in (1, 17, 300, 129, 64, 2000):
        reqs.append(Request("d", rng.uniform(-0.9, 0.9, (P, fleet["d"].d_in)), op="grad",
                            cotangent=rng.normal(size=(P, fleet["d"].d_out)).astype(np.float32)))
    for P in (5, 700, 33, 128):
        reqs.append(Request("d", rng.uniform(-0.9, 0.9, (P, fleet["d"].d_in))))
    for P in (3, 90, 400):
        reqs.append(Request("b", rng.uniform(-0.9, 0.9, (P, fleet["b"].d_in)), precision="fp64"))
    # one stream class (fast_work = 0: no launch is small), so that each group is one launch
    server = Server(fleet, memory_budget=4.0, n_streams=8, staging=1e-5, fast_work=0)  # 10 KiB arena
    for r in reqs:
        server.submit(r)
    server.drain()
    st = server.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["launches"] == 3 and st["batch_launches"] == 3 and st["staging_spills"] > 0
    for r in reqs:
        assert r.error is None
        x = torch.as_tensor(r.x, device="cuda")
        ip = fleet[r.name]
        if r.op == "grad":
            g = torch.as_tensor(r.cotangent, device="cuda")
            alone = ip.spectral_plan().vjp(x, g, need_x=True, need_coef=False)[0].cpu().numpy()
        else:
            alone = ip(x, precision=r.precision).cpu().numpy()
        np.testing.assert_array_equal(r.result, alone)
