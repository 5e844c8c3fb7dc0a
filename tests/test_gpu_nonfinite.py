"""Non-finite query coordinates.

In the reference's barycentric evaluation (``barycentric.py:34-66,117``) a NaN
coordinate gives NaN weights, and an infinite one makes every weight
w_j / (x - node_j) vanish, so the normalisation is 0/0: either way the
point's value is NaN.  Every evaluation path here must do the same for points
with a non-finite coordinate in an active dimension, and leave the other
points' values unchanged (same kernels on the same finite inputs: identical).
"""
import numpy as np
import pytest

import functions as fns

pytestmark = pytest.mark.gpu


def _case(d_out, kind):
    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes

    d = 40
    k = np.log((2 + np.arange(d)) / np.log(2))
    gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
    f = fns.rational_vec(d, d_out, seed=3) if kind == "leja" else fns.exponential(d, d_out, seed=3)
    ip = SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=6.5, d_out=d_out, f=f)
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (300, d)) if kind == "leja" else rng.normal(size=(300, d)) / np.sqrt(2)
    active = np.nonzero(np.asarray(ip._maxdeg) > 0)[0]
    bad = {3: (active[0], np.nan), 7: (active[-1], np.nan), 11: (active[1], np.inf), 13: (active[-2], -np.inf),
           200: (active[len(active) // 2], np.nan)}
    xb = x.copy()
    for p, (j, v) in bad.items():
        xb[p, j] = v
    return ip, x, xb, sorted(bad)


@pytest.mark.parametrize("d_out,kind,path", [(1, "leja", "blocked"), (3, "gh", "perpoint"), (20, "gh", "tensor"),
                                             (1, "gh", "fp64"), (3, "leja", "fp64")])
def test_nonfinite_coordinates_give_nan_rows(d_out, kind, path):
    ip, x, xb, bad = _case(d_out, kind)
    sp = ip.spectral_plan()
    prec = "fp64" if path == "fp64" else "fp32"
    if path == "blocked":
        assert sp.blocked is not None
    elif path == "perpoint":
        assert sp.blocked is None and sp.tc is None
    elif path == "tensor":
        assert sp.tc is not None
    clean = ip(x, precision=prec).cpu().numpy()
    got = ip(xb, precision=prec).cpu().numpy()
    good = np.setdiff1d(np.arange(x.shape[0]), bad)
    assert np.all(np.isnan(got[bad])), "points with a non-finite coordinate must evaluate to NaN"
    assert np.all(np.isfinite(got[good]))
    np.testing.assert_array_equal(got[good], clean[good])
