"""Node rules (host, FP64): values against the oracle's restatement, the
reference's own node test (``tests/test_nodes.py``: sample shapes and
scale/scale_back round trips), and the error types of the drop-in API."""
import numpy as np
import pytest

from oracle import nodes as onodes
from smolyax_gb300 import nodes


def test_leja_sequence_and_weights_match_oracle():
    for n in (0, 1, 2, 4, 5, 9, 17, 40):
        np.testing.assert_array_equal(nodes.Leja1D()(n), onodes.leja_reference_nodes(n))
    for n in range(0, 16):
        np.testing.assert_allclose(nodes.Leja1D().get_quadrature_weights(n),
                                   onodes.rule_quadrature_weights(("leja", None), n), rtol=0, atol=1e-15)
        assert abs(nodes.Leja1D().get_quadrature_weights(n).sum() - 1.0) < 1e-13


def test_leja_custom_domain_nodes_match_oracle():
    dom = (-0.3, 2.5)
    for n in (3, 8):
        np.testing.assert_array_equal(nodes.Leja1D(dom)(n), onodes.rule_nodes(("leja", dom), n))
    gen = nodes.Leja(domains=[(-0.3, 2.5), (1.0, 4.0)])
    np.testing.assert_array_equal(gen[1](6), onodes.rule_nodes(("leja", (1.0, 4.0)), 6))


def test_gauss_hermite_nodes_and_weights_match_oracle():
    for n in (0, 3, 8):
        np.testing.assert_array_equal(nodes.GaussHermite1D()(n), onodes.rule_nodes(("gh", (0.0, 1.0)), n))
        np.testing.assert_array_equal(nodes.GaussHermite1D(0.5, 2.0)(n), onodes.rule_nodes(("gh", (0.5, 2.0)), n))
        np.testing.assert_allclose(nodes.GaussHermite1D().get_quadrature_weights(n),
                                   onodes.rule_quadrature_weights(("gh", (0.0, 1.0)), n), rtol=1e-15)
    gen = nodes.GaussHermite(mean=[0.0, 1.0], scaling=[1.0, 3.0])
    np.testing.assert_array_equal(gen[1](4), onodes.rule_nodes(("gh", (1.0, 3.0)), 4))


def _generators(rng):
    yield nodes.Leja(dim=3)
    yield nodes.GaussHermite(dim=2)
    lo = rng.uniform(-3, 1, 5)
    yield nodes.Leja(domains=np.stack([lo, lo + rng.uniform(0.5, 4, 5)], axis=1))
    yield nodes.GaussHermite(mean=rng.normal(size=4), scaling=rng.uniform(0.5, 2, 4))
    yield nodes.GaussHermite(scaling=[2.0, 0.5])


@pytest.mark.parametrize("n", [0, 1, 3])
def test_random_samples_shape_and_round_trip(n):
    np.random.seed(7)
    for gen in _generators(np.random.default_rng(3)):
        x = gen.get_random(n)
        assert x.shape == ((gen.dim,) if n == 0 else (n, gen.dim))
        np.testing.assert_allclose(gen.scale(gen.scale_back(x)), x, rtol=1e-12, atol=1e-12)


def test_leja_samples_inside_domains():
    np.random.seed(1)
    gen = nodes.Leja(domains=[(2.0, 3.0), (-5.0, -4.0)])
    x = gen.get_random(1000)
    assert np.all((x[:, 0] >= 2) & (x[:, 0] <= 3) & (x[:, 1] >= -5) & (x[:, 1] <= -4))
    ref = gen.scale_back(x)
    assert np.all(np.abs(ref) <= 1 + 1e-12)


def test_errors():
    with pytest.raises(ValueError):
        nodes.Leja()
    with pytest.raises(ValueError):
        nodes.GaussHermite()
    gen = nodes.Leja(domains=[(0.0, 1.0), (0.0, 2.0)])
    with pytest.raises(AssertionError):
        gen.scale(np.array([[0.0, 1.5]]))  # reference coordinates must lie in [-1, 1]
    with pytest.raises(AssertionError):
        gen.scale(np.zeros((4, 3)))  # wrong number of coordinates
    with pytest.raises(AssertionError):
        nodes.Leja1D((0.0, 1.0)).scale(np.array([-2.0]))
    with pytest.raises(AssertionError):
        nodes.Leja(domains=[(1.0, 0.0)])
    with pytest.raises(AssertionError):
        nodes.Generator([nodes.Leja1D(), nodes.GaussHermite1D()])
    # no domain: identity maps
    x = np.array([0.25, -0.5])
    assert nodes.Leja(dim=2).scale(x) is x
    assert nodes.Leja1D().scale_back(x) is x


def test_generator_container_interface():
    gen = nodes.GaussHermite(mean=[0.0, 1.0, 2.0])
    assert gen.dim == 3 and len(gen) == 3 and not gen.is_nested
    assert [g.mean for g in gen] == [0.0, 1.0, 2.0]
    assert nodes.Leja(dim=4).is_nested
    lj = nodes.Leja1D((-2.0, 2.0))
    assert lj.spectral_map() == ("legendre", 0.5, 0.0)
    assert nodes.GaussHermite1D(1.0, 2.0).spectral_map() == ("hermite", 0.5, -0.5)
    assert "Leja" in repr(nodes.Leja(dim=2)) and "GaussHermite" in repr(gen)
