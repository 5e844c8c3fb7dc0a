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


def check_fp64(y, ref, exact, tol=1e-12, what="values"):
    """FP64 parity contract.  The combination sum cancels strongly, so the
    reference's own FP64 output is off from the exact value of its FP64 data by
    up to 1e-10 on some workloads; no FP64 evaluation can be within 1e-12 of it
    there.  The contract is: our max relative error against the
    extended-precision value of the same data is at most max(tol, the
    reference's own max relative error)."""
    y, ref, exact = (np.asarray(v, dtype=float) for v in (y, ref, exact))
    e_ours, e_ref = rel_err(y, exact), rel_err(ref, exact)
    print("FP64 %s: max rel err ours %.3e, reference %.3e (vs extended precision)" % (what, e_ours, e_ref))
    assert e_ours <= max(tol, e_ref), "ours %.3e, reference %.3e" % (e_ours, e_ref)


def check_fp64_grad(g, ref, exact, tol=2e-12):
    """Gradients: the same contract norm-wise (gradients have tiny components)."""
    g, ref, exact = (np.asarray(v, dtype=float) for v in (g, ref, exact))
    scale = float(np.max(np.abs(exact)))
    e_ours = float(np.max(np.abs(g - exact))) / scale
    e_ref = float(np.max(np.abs(ref - exact))) / scale
    print("FP64 gradient: norm-wise rel err ours %.3e, reference %.3e" % (e_ours, e_ref))
    assert e_ours <= max(tol, e_ref), "ours %.3e, reference %.3e" % (e_ours, e_ref)
