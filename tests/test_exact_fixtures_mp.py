"""A second, independent check of the extended-precision fixtures.

``tests/golden/exact_configs.npz`` holds the combination sum of the benchmark
configurations evaluated in numpy ``longdouble`` (80-bit extended precision)
by ``tests/golden/make_exact.py``; the FP64 parity tests compare the GPU FP64
path with those values at 1e-12 (or the reference's own error when that is
larger).  Here the same formula -- FP64 nodes, FP64 nodal values, FP64 query
points, barycentric weights and basis recomputed from the nodes -- is
evaluated once more in mpmath at 40 significant digits, summand by summand
from the oracle's blocks (``interpolation.py:264-304``,
``barycentric.py:13-31,34-66,69-123``), on a few points of each
configuration.  The fixtures must agree with it to 1e-14 relative: the
combination sum cancels terms up to ~2e4 times the result, so 64-bit
mantissas leave ~1e-15, a hundred times below the bounds the fixtures serve.
"""
import numpy as np
import pytest

import functions as fns
import golden_io as gio
from oracle import interp as ointerp

mpmath = pytest.importorskip("mpmath")

EXACT = gio.load("exact_configs.npz")


def _basis(xv, xi):
    """Normalised barycentric basis at xv (one-hot at an exact node)."""
    g = len(xi)
    w = [mpmath.fprod([1 / (xi[a] - xi[b]) for a in range(g) if xi[a] != xi[b]]) for b in range(g)]
    hits = [j for j in range(g) if xv == xi[j]]
    if hits:
        return [mpmath.mpf(1) / len(hits) if j in hits else mpmath.mpf(0) for j in range(g)]
    b = [w[j] / (xv - xi[j]) for j in range(g)]
    S = mpmath.fsum(b)
    return [v / S for v in b]


def _contract(T, Ls, s):
    if s == len(Ls):
        return mpmath.mpf(float(T))
    return mpmath.fsum(Ls[s][j] * _contract(T[j], Ls, s + 1) for j in range(len(Ls[s])))


def mp_values(ip, x):
    """The combination sum at one point x (FP64), every output, in mpmath."""
    X = [mpmath.mpf(float(v)) for v in x]
    off = np.broadcast_to(np.asarray(ip.offset, dtype=float), (ip.d_out,))
    total = [mpmath.mpf(float(v)) for v in off]
    for n, blk in ip.blocks.items():
        dims, degs, nodes, zetas, F = blk["dims"], blk["degs"], blk["nodes"], blk["zetas"], blk["F"]
        for z in range(zetas.shape[0]):
            Ls = []
            for s in range(n):
                g = int(degs[z, s])
                Ls.append(_basis(X[int(dims[z, s])], [mpmath.mpf(float(v)) for v in nodes[z, s, : g + 1]]))
            for o in range(ip.d_out):
                total[o] += int(zetas[z]) * _contract(F[z, o], Ls, 0)
    return total


CASES = {
    # tag: (d, t, kind, d_out, f, x generator, points checked)
    "cfg1": (10, 8.831421, "leja", 1, lambda: fns.rational(10, seed=0),
             lambda: np.random.default_rng(1).uniform(-1, 1, (10000, 10)), [0, 1, 2]),
    "cfg2": (1000, 8.224520, "leja", 1, lambda: fns.rational(1000, seed=0),
             lambda: np.random.default_rng(1).uniform(-1, 1, (256, 1000)), [0]),
    "cfg3alt": (100, 7.723434, "gh", 8, lambda: fns.exponential(100, 8, seed=0),
                lambda: np.random.default_rng(1).normal(size=(32, 100)), [0]),
}


@pytest.mark.parametrize("tag", list(CASES))
def test_longdouble_fixtures_against_mpmath(tag):
    d, t, kind, d_out, f, xgen, pts = CASES[tag]
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = ointerp.OracleInterpolant(rules=ointerp.rules_from_spec(kind, d), k=k, t=t, d_out=d_out, f=f(),
                                   nested=(kind == "leja"))
    x = xgen()
    y = np.asarray(EXACT[tag + "/y"], dtype=float).reshape(x.shape[0], d_out)
    with mpmath.workdps(40):
        for i in pts:
            ref = mp_values(ip, x[i])
            for o in range(d_out):
                err = abs(mpmath.mpf(float(y[i, o])) - ref[o]) / abs(ref[o])
                assert err < 1e-14, (tag, i, o, float(err))
