"""The CPU oracle against the reference's own outputs and known answers.

Golden vectors come from running the reference itself
(``tests/golden/make_golden.py``); the cardinality pins 98 / 1000 / 10003 are
the reference's runtime-test pins.  Index sets, coefficients and their DFS
order must match exactly; interpolant values within 1e-12 relative.
"""
import numpy as np
import pytest

import functions as fns
import golden_io as gio
from oracle import indices as oi
from oracle import interp as ointerp


def _close(a, b, rtol=1e-12, atol=1e-13):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    assert a.shape == b.shape, (a.shape, b.shape)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(a)
    np.testing.assert_allclose(a[m], b[m], rtol=rtol, atol=atol)


SMALL = gio.load("indices_small.npz")


@pytest.mark.parametrize("name", [str(n) for n in SMALL["names"]])
def test_indices_small(name):
    z = SMALL
    k, t = z[name + "/k"], float(z[name + "/t"])
    iset = gio.unflatten(z[name + "/iset_lens"], z[name + "/iset_dims"], z[name + "/iset_degs"])
    assert oi.indexset(k, t) == iset
    card = [oi.indexset_cardinality(k, t), oi.nodeset_cardinality(k, t, True), oi.nodeset_cardinality(k, t, False)]
    assert card == [int(v) for v in z[name + "/card"]]
    coef = [oi.smolyak_coefficient(k, len(k), r, 0) for r in z[name + "/coef_rem"]]
    assert coef == [int(v) for v in z[name + "/coef"]]
    n2nus, n2z = oi.non_zero_indices_and_zetas(k, t)
    assert list(n2nus.keys()) == [int(v) for v in z[name + "/nz_n_keys"]]
    nus, zetas = gio.nonzero_list(z, name + "/")
    assert [nu for n in n2nus for nu in n2nus[n]] == nus
    assert [v for n in n2z for v in n2z[n]] == zetas
    n_t, nested = (int(v) for v in z[name + "/target"])
    if n_t > 0:
        assert oi.find_approximate_threshold(k, n_t, nested=bool(nested)) == t


CONFIGS = gio.load("indices_configs.npz")


@pytest.mark.parametrize("name", ["cfg1", "cfg2", "cfg3", "cfg3alt", "cfg4"])
def test_indices_configs(name):
    z = CONFIGS
    d, t = int(z[name + "/d"]), float(z[name + "/t"])
    k = np.log((2 + np.arange(d)) / np.log(2))
    n2nus, n2z = oi.non_zero_indices_and_zetas(k, t)
    nus, zetas = gio.nonzero_list(z, name + "/")
    assert [nu for n in n2nus for nu in n2nus[n]] == nus
    assert [v for n in n2z for v in n2z[n]] == zetas
    card = [oi.indexset_cardinality(k, t), oi.nodeset_cardinality(k, t, True), oi.nodeset_cardinality(k, t, False)]
    assert card == [int(v) for v in z[name + "/card"]]


def test_cardinality_pins_d10000():
    k = np.log([2 + i for i in range(10000)]) / np.log(2)
    for t, m_len, m_card in CONFIGS["pins_d10000"]:
        assert (int(m_len), int(m_card)) in ((98, 98), (1000, 1000), (10003, 10003))
        assert oi.indexset_cardinality(k, t) == int(m_card)


def test_thresholds():
    for d, m, nested, acc, t_ref, card in CONFIGS["thresholds"]:
        d, m = int(d), int(m)
        k = np.log([2 + i for i in range(d)]) / np.log(2)
        t = oi.find_approximate_threshold(k, m, nested=bool(nested), accuracy=acc)
        assert t == t_ref
        assert oi.nodeset_cardinality(k, t, nested=bool(nested)) == int(card)


INTERP = gio.load("interp_small.npz")


def _oracle_from_spec(spec, k, t, d_out, f):
    d = len(k)
    if spec["kind"] == "leja":
        rules = ointerp.rules_from_spec("leja", d, domains=spec["domains"])
        nested = True
    else:
        rules = ointerp.rules_from_spec("gh", d, mean=spec["mean"], scaling=spec["scaling"])
        nested = False
    return ointerp.OracleInterpolant(rules=rules, k=k, t=t, d_out=d_out, f=f, nested=nested)


@pytest.mark.parametrize("name", [str(n) for n in INTERP["names"]])
def test_interp_small(name):
    z = INTERP
    spec, k, t, d_out, f = gio.small_case(z, name)
    ip = _oracle_from_spec(spec, k, t, d_out, f)
    x = z[name + "/x"]
    _close(ip(x), z[name + "/y"])
    _close(ip.gradient(x[:-1]), z[name + "/grad"], rtol=1e-10, atol=1e-11)
    _close(ip.integral(), z[name + "/integral"], atol=1e-12)
    assert ip.n_f_evals_new == int(z[name + "/n_f_evals"][1])
    # known answer: the interpolant reproduces polynomials of the index set
    np.testing.assert_allclose(ip(x), f(x), rtol=1e-7, atol=1e-8)
    np.testing.assert_allclose(ip.integral(), f.integral(), atol=1e-8)


def test_exact_node_gradient_is_nan():
    """At an interpolation node the reference's gradient is NaN in that dimension."""
    ip = ointerp.OracleInterpolant(rules=[("leja", None)] * 2, k=[1.0, 1.5], t=3.2, d_out=1,
                                   f=lambda x: np.array([np.sin(x[0]) + x[1] ** 2]), nested=True)
    g = ip.gradient(np.array([[0.0, 0.3]]))
    assert np.isnan(g[0, 0, 0]) and np.isfinite(g[0, 0, 1])
