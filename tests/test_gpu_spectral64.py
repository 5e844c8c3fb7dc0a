"""FP64 evaluator of the orthogonal form (``csrc/spectral64.cu``).

It is what ``ip(x)`` runs for Leja / Gauss-Hermite plans.  Bounds:
against the extended-precision values of the benchmark workloads (cfg1,
cfg2) 1e-13 element-wise relative -- tighter than the FP64 contract of
``gpu_helpers.check_fp64`` (1e-12, or the reference's own error), because the
form sums terms of the size of the result (the combination sum's cancellation
is taken by compensated sums once, in the coefficients); against the
barycentric FP64 evaluator 1e-12 element-wise on rules, domains, partial and
multi-tile point counts (1e-11 for Gauss-Hermite plans with several outputs,
where the combination sum itself is off by up to that much).  Non-finite
coordinates: NaN / Inf in an active dimension gives NaN for that point only;
inactive dimensions are never read.  Plans with several outputs run four
outputs per pass.  The tables are checked to select this evaluator
(``_fp64_orthogonal``).
"""
import numpy as np
import pytest
import torch

import functions as fns
import golden_io as gio
from gpu_helpers import rel_err

pytestmark = pytest.mark.gpu

EXACT = gio.load("exact_configs.npz")
BARY = "fp64_barycentric"


def _interp(**kw):
    from smolyax_gb300 import SmolyakBarycentricInterpolator

    return SmolyakBarycentricInterpolator(**kw)


@pytest.fixture(scope="module")
def cfg2():
    from smolyax_gb300 import nodes

    d = 1000
    k = np.log((2 + np.arange(d)) / np.log(2))
    return _interp(node_gen=nodes.Leja(dim=d), k=k, t=8.224520, d_out=1, f=fns.rational(d, seed=0))


@pytest.mark.parametrize("tag", ["cfg1", "cfg2"])
def test_against_extended_precision(tag, cfg2):
    from smolyax_gb300 import nodes

    if tag == "cfg2":
        ip, x = cfg2, np.random.default_rng(1).uniform(-1, 1, (256, 1000))
    else:
        d = 10
        k = np.log((2 + np.arange(d)) / np.log(2))
        ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=8.831421, d_out=1, f=fns.rational(d, seed=0))
        x = np.random.default_rng(1).uniform(-1, 1, (10000, d))
    assert ip._fp64_orthogonal() is not None
    exact = np.asarray(EXACT[tag + "/y"], dtype=float).reshape(-1)
    y = ip(x).cpu().numpy()[:, 0]
    yb = ip(x, precision=BARY).cpu().numpy()[:, 0]
    e, eb = rel_err(y, exact), rel_err(yb, exact)
    print("%s: orthogonal FP64 %.3e, barycentric FP64 %.3e (element-wise vs extended precision, bound 1e-13)"
          % (tag, e, eb))
    assert e < 1e-13


@pytest.mark.parametrize("P", [1, 127, 129, 20000])
def test_points_and_tiles(P, cfg2):
    x = np.random.default_rng(P).uniform(-1, 1, (P, 1000))
    y = cfg2(x).cpu().numpy()
    yb = cfg2(x, precision=BARY).cpu().numpy()
    err = rel_err(y, yb)
    print("cfg2, %d points: orthogonal vs barycentric FP64 %.3e (bound 1e-12)" % (P, err))
    assert y.shape == (P, 1) and err < 1e-12


@pytest.mark.parametrize("kind,d,t", [("leja", 200, 6.5), ("leja_domain", 120, 6.2), ("gh", 60, 5.8),
                                      ("gh_scaled", 40, 6.0), ("leja", 3, 14.0),
                                      ("leja", 1, 30.0), ("gh", 2, 26.0)])
def test_rules_and_domains(kind, d, t):
    from smolyax_gb300 import nodes

    k = np.log((2 + np.arange(d)) / np.log(2))
    rng = np.random.default_rng(d)
    if kind == "leja":
        gen, x, f = nodes.Leja(dim=d), rng.uniform(-1, 1, (700, d)), fns.rational(d, seed=2)
    elif kind == "leja_domain":
        dom = np.stack([np.linspace(-2.0, 0.5, d), np.linspace(1.0, 3.5, d)], axis=1)
        gen = nodes.Leja(domains=dom)
        x = rng.uniform(dom[:, 0], dom[:, 1], (700, d))
        w = fns.rational(d, seed=2).w
        mid = dom.mean(axis=1)
        half = (dom[:, 1] - dom[:, 0]) / 2

        def f(z):
            z = np.asarray(z, dtype=float)
            u = (z - mid) / half
            return np.atleast_1d(1.0 / (1.0 + u @ w)) if z.ndim == 1 else (1.0 / (1.0 + u @ w))[:, None]
    elif kind == "gh":
        gen, x, f = nodes.GaussHermite(dim=d), rng.normal(size=(700, d)), fns.exponential(d, 1, seed=2)
    else:
        mean, scale = rng.uniform(-1, 1, d), rng.uniform(0.5, 2.0, d)
        gen = nodes.GaussHermite(mean, scale)
        x = mean + scale * rng.normal(size=(700, d))
        A = fns.exponential(d, 1, seed=2).A

        def f(z):
            z = np.asarray(z, dtype=float)
            return np.exp(-(((z - mean) / scale) @ A.T)) if z.ndim == 2 else np.exp(-(A @ ((z - mean) / scale)))
    ip = _interp(node_gen=gen, k=k, t=t, d_out=1, f=f)
    assert ip._fp64_orthogonal() is not None
    y = ip(x).cpu().numpy()
    yb = ip(x, precision=BARY).cpu().numpy()
    err = rel_err(y, yb)
    print("%s d=%d t=%.1f: orthogonal vs barycentric FP64 %.3e (bound 1e-12)" % (kind, d, t, err))
    assert err < 1e-12


def test_nodes_nonfinite_and_inactive():
    """At grid points the value is the nodal value (to rounding); NaN / Inf in
    an active coordinate makes that point NaN and leaves the others unchanged;
    inactive dimensions (degree 0 everywhere) are not read."""
    from smolyax_gb300 import nodes

    d = 200
    k = np.log((2 + np.arange(d)) / np.log(2))
    f = fns.rational(d, seed=4)
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=4.5, d_out=1, f=f)
    assert ip._fp64_orthogonal() is not None
    active = np.nonzero(np.asarray(ip._maxdeg) > 0)[0]
    inactive = np.setdiff1d(np.arange(d), active)
    assert inactive.size > 0
    # grid points: one coordinate at its dimension's degree-1 node (1), the rest at node 0 (0)
    assert list(nodes.Leja(dim=1)[0](1)) == [0.0, 1.0]
    xg = np.zeros((len(active), d))
    xg[np.arange(len(active)), active] = 1.0
    yg = ip(xg).cpu().numpy()[:, 0]
    fg = np.array([f(v)[0] for v in xg])
    assert rel_err(yg, fg) < 1e-14
    x = np.random.default_rng(5).uniform(-1, 1, (300, d))
    clean = ip(x).cpu().numpy()[:, 0]
    xi = x.copy()
    xi[:, inactive[:3]] = np.nan
    xi[::2, inactive[-1]] = np.inf
    np.testing.assert_array_equal(ip(xi).cpu().numpy()[:, 0], clean)
    bad = {5: (active[0], np.nan), 17: (active[-1], np.inf), 40: (active[1], -np.inf), 299: (active[2], np.nan)}
    xb = x.copy()
    for p, (j, v) in bad.items():
        xb[p, j] = v
    got = ip(xb).cpu().numpy()[:, 0]
    rows = sorted(bad)
    good = np.setdiff1d(np.arange(300), rows)
    assert np.all(np.isnan(got[rows]))
    np.testing.assert_array_equal(got[good], clean[good])


def test_device_input_strides_and_dispatch():
    """Device FP64 inputs (contiguous or not) give the same values."""
    from smolyax_gb300 import nodes

    d = 50
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=6.0, d_out=1, f=fns.rational(d, seed=7))
    x = np.random.default_rng(7).uniform(-1, 1, (1000, d))
    y_host = ip(x).cpu().numpy()
    xd = torch.as_tensor(np.concatenate([x, x], axis=1), device="cuda")[:, :d]
    np.testing.assert_array_equal(ip(xd).cpu().numpy(), y_host)


@pytest.mark.parametrize("kind,d,t,d_out", [("leja", 30, 6.0, 2), ("leja", 60, 6.5, 7), ("gh", 40, 6.0, 9),
                                            ("leja", 12, 7.0, 64)])
def test_several_outputs(kind, d, t, d_out):
    """Several outputs (four per pass, the last pass partial): against the
    barycentric FP64 evaluator at 1e-12 element-wise for Leja plans, 1e-11 for
    Gauss-Hermite ones, whose combination sum itself cancels to 1e-12 .. 1e-11
    (measured against extended precision at the benchmark configurations)."""
    from smolyax_gb300 import nodes

    k = np.log((2 + np.arange(d)) / np.log(2))
    rng = np.random.default_rng(d_out)
    if kind == "leja":
        gen, x, f = nodes.Leja(dim=d), rng.uniform(-1, 1, (333, d)), fns.rational_vec(d, d_out, seed=3)
    else:
        gen, x, f = nodes.GaussHermite(dim=d), rng.normal(size=(333, d)), fns.exponential(d, d_out, seed=3)
    ip = _interp(node_gen=gen, k=k, t=t, d_out=d_out, f=f)
    assert ip._fp64_orthogonal() is not None
    y = ip(x).cpu().numpy()
    yb = ip(x, precision=BARY).cpu().numpy()
    err = rel_err(y, yb)
    bound = 1e-12 if kind == "leja" else 1e-11
    print("%s d=%d d_out=%d: orthogonal vs barycentric FP64 %.3e (bound %.0e)" % (kind, d, d_out, err, bound))
    assert y.shape == (333, d_out) and err < bound
