"""Tensor-core blocked evaluator (one output, ``csrc/blocked_tc.cu``).

Norm and bound as for the blocked evaluator (``test_gpu_spectral.py``):
element-wise relative error max_p |y32 - y64| / |y64| <= 1e-6 against the
extended-precision values (cfg1, cfg2) or the FP64 path; the two FP32
evaluators are also compared with each other.  Gauss-Hermite cases are held
to 1e-6 relative to sum_m |c_m phi_m(x)| (the size of what FP32 sums; the
element-wise error is printed).  Further cases: a shifted domain (the folded
constant column), partial and single-point tiles, inactive dimensions
(masked units of 8 columns: their coordinates are never read, NaN there
leaves the value unchanged), non-finite active coordinates (NaN rows, the
other rows unchanged), and the error flag staying clear.
"""
import numpy as np
import pytest
import torch

import functions as fns
import golden_io as gio
from gpu_helpers import rel_err
from test_gpu_spectral import term_relative_error

pytestmark = pytest.mark.gpu

EXACT = gio.load("exact_configs.npz")


def _interp(**kw):
    from smolyax_gb300 import SmolyakBarycentricInterpolator

    return SmolyakBarycentricInterpolator(**kw)


def _eval(ip, x, mode):
    sp = ip.spectral_plan()
    xt = torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")
    y = torch.empty(xt.shape[0], 1, dtype=torch.float32, device="cuda")
    sp.evaluate(xt, y, mode=mode)
    return y.cpu().numpy()[:, 0].astype(float)


def _flag(ip):
    return int(ip.spectral_plan().blocked_tc_keep[0]["err"].item())


@pytest.fixture(scope="module")
def cfg2():
    from smolyax_gb300 import nodes

    d = 1000
    k = np.log((2 + np.arange(d)) / np.log(2))
    return _interp(node_gen=nodes.Leja(dim=d), k=k, t=8.224520, d_out=1, f=fns.rational(d, seed=0))


@pytest.mark.parametrize("tag", ["cfg1", "cfg2"])
def test_exact_configs(tag, cfg2):
    """cfg1 (d = 10: table dimensions only) and cfg2 (d = 1000: 41 table and
    959 linear dimensions) against their extended-precision values."""
    from smolyax_gb300 import nodes

    if tag == "cfg2":
        ip, x = cfg2, np.random.default_rng(1).uniform(-1, 1, (256, 1000))
    else:
        d = 10
        k = np.log((2 + np.arange(d)) / np.log(2))
        ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=8.831421, d_out=1, f=fns.rational(d, seed=0))
        x = np.random.default_rng(1).uniform(-1, 1, (10000, d))
    assert ip.spectral_plan().blocked_tc is not None
    y_tc = _eval(ip, x, "blocked_tc")
    y_bl = _eval(ip, x, "blocked")
    exact = np.asarray(EXACT[tag + "/y"], dtype=float).reshape(-1)
    e_tc, e_bl = rel_err(y_tc, exact), rel_err(y_bl, exact)
    print("%s: tensor-core blocked %.3e, blocked %.3e (element-wise vs exact, bound 1e-06); between them %.3e"
          % (tag, e_tc, e_bl, rel_err(y_tc, y_bl)))
    assert e_tc < 1e-6 and rel_err(y_tc, y_bl) < 1e-6
    assert _flag(ip) == 0


@pytest.mark.parametrize("P", [1, 129, 1000, 20000])
def test_points_and_tiles(P, cfg2):
    """Partial tiles, fewer tiles than SMs and more: against the FP64 path."""
    x = np.random.default_rng(P).uniform(-1, 1, (P, 1000))
    y64 = cfg2(x).cpu().numpy()[:, 0]
    y_tc = _eval(cfg2, x, "blocked_tc")
    err = rel_err(y_tc, y64)
    print("cfg2, %d points: element-wise %.3e (bound 1e-06)" % (P, err))
    assert err < 1e-6 and _flag(cfg2) == 0


@pytest.mark.parametrize("kind,d,t", [("leja", 200, 6.5), ("leja_shifted", 120, 6.2), ("gh", 60, 5.8),
                                      ("gh", 100, 7.723434)])
def test_rules_and_domains(kind, d, t):
    from smolyax_gb300 import nodes

    k = np.log((2 + np.arange(d)) / np.log(2))
    rng = np.random.default_rng(d)
    if kind == "leja":
        gen, x, f = nodes.Leja(dim=d), rng.uniform(-1, 1, (700, d)), fns.rational(d, seed=2)
    elif kind == "leja_shifted":
        dom = np.stack([np.full(d, 0.5), np.full(d, 2.5)], axis=1)
        gen, x = nodes.Leja(domains=dom), rng.uniform(0.5, 2.5, (700, d))
        w = fns.rational(d, seed=2).w

        def f(z):
            z = np.asarray(z, dtype=float)
            return np.atleast_1d(1.0 / (1.0 + (z - 1.5) @ w)) if z.ndim == 1 else (1.0 / (1.0 + (z - 1.5) @ w))[:, None]
    else:
        gen, x, f = nodes.GaussHermite(dim=d), rng.normal(size=(700, d)), fns.exponential(d, 1, seed=2)
    ip = _interp(node_gen=gen, k=k, t=t, d_out=1, f=f)
    sp = ip.spectral_plan()
    if sp.blocked_tc is None:
        pytest.skip("plan outside the tensor-core blocked evaluator's limits")
    y64 = ip(x).cpu().numpy()[:, 0]
    y_tc = _eval(ip, x, "blocked_tc")
    ew = rel_err(y_tc, y64)
    tr = term_relative_error(ip, x, y_tc[:, None], y64[:, None])
    print("%s d=%d: element-wise %.3e, relative to sum|terms| %.3e" % (kind, d, ew, tr))
    assert tr < 1e-6
    if kind != "gh":
        assert ew < 1e-6
    assert _flag(ip) == 0


def test_inactive_and_nonfinite_coordinates():
    """d = 200, t = 4.5: dimensions 0..60 are active, the x boxes cover 0..63,
    so 61..63 are masked.  NaN / Inf in an inactive dimension (masked, or
    beyond the boxes) leaves the value unchanged; in an active table or linear
    dimension it gives NaN, the other rows equal the clean evaluation."""
    from smolyax_gb300 import nodes

    d = 200
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=4.5, d_out=1, f=fns.rational(d, seed=4))
    sp = ip.spectral_plan()
    assert sp.blocked_tc is not None
    lin0, nb = int(sp.blocked_tc.lin0), int(sp.blocked_tc.n_boxes)
    active = np.nonzero(ip._maxdeg > 0)[0]
    assert active.max() == 60 and lin0 + 8 * nb == 64
    x = np.random.default_rng(5).uniform(-1, 1, (300, d))
    clean = _eval(ip, x, "blocked_tc")
    assert rel_err(clean, ip(x).cpu().numpy()[:, 0]) < 1e-6
    xi = x.copy()
    xi[::3, 62] = np.nan
    xi[1::3, 63] = np.inf
    xi[2::3, 150] = np.nan
    np.testing.assert_array_equal(_eval(ip, xi, "blocked_tc"), clean)
    bad = {5: (1, np.nan), 17: (60, np.nan), 40: (33, -np.inf), 299: (0, np.inf)}
    xb = x.copy()
    for p, (j, v) in bad.items():
        xb[p, j] = v
    got = _eval(ip, xb, "blocked_tc")
    rows = sorted(bad)
    good = np.setdiff1d(np.arange(300), rows)
    assert np.all(np.isnan(got[rows]))
    np.testing.assert_array_equal(got[good], clean[good])
    assert _flag(ip) == 0

