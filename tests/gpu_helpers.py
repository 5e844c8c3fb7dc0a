"""Builders shared by the GPU tests."""
import numpy as np


def product_generator(spec, d):
    from smolyax_gb300 import nodes

    if spec["kind"] == "leja":
        return nodes.Leja(domains=spec["domains"]) if spec["domains"] is not None else nodes.Leja(dim=d)
    if spec.get("mean") is None:
        return nodes.GaussHermite(dim=d)
    return nodes.GaussHermite(spec["mean"], spec["scaling"])


def rel_err(a, b, floor=1e-300):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


def assert_close_nan(a, b, rtol, atol):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    assert a.shape == b.shape, (a.shape, b.shape)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(a)
    np.testing.assert_allclose(a[m], b[m], rtol=rtol, atol=atol)
