"""Backward of the mixed-precision form behind torch.autograd.

dL/dx is checked against central finite differences of the FP64 path
(h = 1e-6) and against the reference's own derivative (the FP64 Jacobian of
``gradient`` contracted with the cotangent); dL/d(nodal values) against
central differences through ``set_nodal_values`` (the interpolant is linear
in them, so the difference quotient is exact up to rounding).  Bound: 1e-5
norm-wise (the forward and the products run in FP32 / 3xTF32).
"""
import numpy as np
import pytest
import torch

import functions as fns

pytestmark = pytest.mark.gpu


def _ip(kind, d, t, d_out, f):
    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes

    k = np.log((2 + np.arange(d)) / np.log(2))
    gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
    return SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=t, d_out=d_out, f=f)


CASES = [
    ("leja", 20, 6.5, 4, lambda d, o: fns.rational_vec(d, o, seed=1)),
    ("gh", 12, 6.0, 3, lambda d, o: fns.exponential(d, o, seed=2)),
    ("leja", 200, 7.853604, 64, lambda d, o: fns.rational_vec(d, o, seed=0)),
]


@pytest.mark.parametrize("kind,d,t,d_out,fb", CASES)
def test_vjp_x(kind, d, t, d_out, fb):
    from smolyax_gb300.autograd import interpolate

    ip = _ip(kind, d, t, d_out, fb(d, d_out))
    rng = np.random.default_rng(5)
    P = 64
    xs = rng.uniform(-0.9, 0.9, (P, d)) if kind == "leja" else rng.normal(size=(P, d))
    x = torch.tensor(xs, device="cuda", requires_grad=True)
    g = torch.tensor(rng.normal(size=(P, d_out)), device="cuda", dtype=torch.float32)
    y = interpolate(ip, x)
    (y * g).sum().backward()
    dx = x.grad.cpu().numpy()
    # reference derivative: FP64 Jacobian contracted with the cotangent
    J = ip.gradient(xs).cpu().numpy()
    ref = np.einsum("po,poj->pj", g.double().cpu().numpy(), J)
    err = np.max(np.abs(dx - ref)) / np.max(np.abs(ref))
    print("%s d=%d d_out=%d: dL/dx vs reference Jacobian %.2e" % (kind, d, d_out, err))
    assert err < 1e-5
    # central differences of the FP64 path in a few coordinates
    h = 1e-6
    gd = g.double().cpu().numpy()
    for j in rng.choice(d, size=min(d, 4), replace=False):
        e = np.zeros(d)
        e[j] = h
        fd = ((ip(xs + e).cpu().numpy() - ip(xs - e).cpu().numpy()) * gd).sum(1) / (2 * h)
        assert np.max(np.abs(fd - dx[:, j])) <= 1e-5 * max(1.0, np.max(np.abs(fd)))


@pytest.mark.parametrize("kind,d,t,d_out,fb", CASES[:2])
def test_vjp_nodal_values(kind, d, t, d_out, fb):
    from smolyax_gb300.autograd import interpolate

    ip = _ip(kind, d, t, d_out, fb(d, d_out))
    rng = np.random.default_rng(6)
    P = 50
    xs = rng.uniform(-0.9, 0.9, (P, d)) if kind == "leja" else rng.normal(size=(P, d))
    fu = ip.nodal_values.clone().requires_grad_(True)
    g = torch.tensor(rng.normal(size=(P, d_out)), device="cuda", dtype=torch.float32)
    y = interpolate(ip, torch.tensor(xs, device="cuda"), fu)
    (y * g).sum().backward()
    dfu = fu.grad
    v = torch.tensor(rng.normal(size=tuple(fu.shape)), device="cuda", dtype=torch.float64)
    base = fu.detach().clone()
    eps = 1e-3
    gd = g.double()
    ip.set_nodal_values(base + eps * v)
    lp = float((ip(xs) * gd).sum())
    ip.set_nodal_values(base - eps * v)
    lm = float((ip(xs) * gd).sum())
    ip.set_nodal_values(base)
    fd = (lp - lm) / (2 * eps)
    got = float((dfu * v).sum())
    print("%s: <dL/dfu, v> %.6e vs central difference %.6e" % (kind, got, fd))
    assert abs(got - fd) <= 1e-5 * max(1.0, abs(fd))
