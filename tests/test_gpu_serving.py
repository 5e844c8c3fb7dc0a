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
