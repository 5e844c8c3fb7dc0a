"""GPU index sets and Smolyak coefficients against the reference's own outputs.

Bit-exact: the same multi-indices in the same order, the same integer
coefficients, the same cardinalities and thresholds.
"""
import numpy as np
import pytest

import golden_io as gio

pytestmark = pytest.mark.gpu

SMALL = gio.load("indices_small.npz")
CONFIGS = gio.load("indices_configs.npz")


@pytest.fixture(scope="module")
def idx():
    from smolyax_gb300 import indices

    return indices


@pytest.mark.parametrize("name", [str(n) for n in SMALL["names"]])
def test_small_sets(idx, name):
    z = SMALL
    k, t = z[name + "/k"], float(z[name + "/t"])
    iset = gio.unflatten(z[name + "/iset_lens"], z[name + "/iset_dims"], z[name + "/iset_degs"])
    assert idx.indexset(k, t) == iset
    card = [idx.indexset_cardinality(k, t), idx.nodeset_cardinality(k, t, True), idx.nodeset_cardinality(k, t, False)]
    assert card == [int(v) for v in z[name + "/card"]]
    n2nus, n2z = idx.non_zero_indices_and_zetas(k, t)
    assert list(n2nus.keys()) == [int(v) for v in z[name + "/nz_n_keys"]]
    nus, zetas = gio.nonzero_list(z, name + "/")
    assert [nu for n in n2nus for nu in n2nus[n]] == nus
    assert [v for n in n2z for v in n2z[n]] == zetas
    rems, coefs = z[name + "/coef_rem"], z[name + "/coef"]
    for r, c in list(zip(rems, coefs))[:12]:
        assert idx.smolyak_coefficient(k, len(k), float(r), 0) == int(c)
        assert idx.smolyak_coefficient(k, len(k), float(r), 1) == -int(c)


@pytest.mark.parametrize("name", ["cfg1", "cfg2", "cfg3", "cfg3alt", "cfg4"])
def test_config_sets(idx, name):
    z = CONFIGS
    d, t = int(z[name + "/d"]), float(z[name + "/t"])
    k = np.log((2 + np.arange(d)) / np.log(2))
    n2nus, n2z = idx.non_zero_indices_and_zetas(k, t)
    nus, zetas = gio.nonzero_list(z, name + "/")
    assert [nu for n in n2nus for nu in n2nus[n]] == nus
    assert [v for n in n2z for v in n2z[n]] == zetas
    card = [idx.indexset_cardinality(k, t), idx.nodeset_cardinality(k, t, True), idx.nodeset_cardinality(k, t, False)]
    assert card == [int(v) for v in z[name + "/card"]]


def test_cardinality_pins_d10000(idx):
    k = np.log([2 + i for i in range(10000)]) / np.log(2)
    for t, m_len, m_card in CONFIGS["pins_d10000"]:
        assert idx.indexset_cardinality(k, float(t)) == int(m_card)
        assert len(idx.indexset(k, float(t))) == int(m_len)


def test_thresholds(idx):
    for d, m, nested, acc, t_ref, card in CONFIGS["thresholds"]:
        k = np.log([2 + i for i in range(int(d))]) / np.log(2)
        t = idx.find_approximate_threshold(k, int(m), nested=bool(nested), accuracy=acc)
        assert t == t_ref
        assert idx.nodeset_cardinality(k, t, nested=bool(nested)) == int(card)


def test_edge_cases(idx):
    # threshold below every weight: Lambda = {0}
    k = [1.0, 2.0]
    assert idx.indexset(k, 0.5) == [()]
    assert idx.indexset_cardinality(k, 0.5) == 1
    n2nus, n2z = idx.non_zero_indices_and_zetas(k, 0.5)
    assert dict(n2nus) == {0: [()]} and dict(n2z) == {0: [1]}
    # one dimension
    assert idx.indexset([1.0], 3.5) == [((0, 3),), ((0, 2),), ((0, 1),), ()]
    assert idx.find_approximate_threshold([1.0, 1.5], 1, nested=True) == 1
