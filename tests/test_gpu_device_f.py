"""Target functions evaluated on the device (``f.on_device``): the same unique
nodes, row map and nodal values as the host path (the same function written
with numpy), so the same interpolant; a wrong output width is an error."""
import numpy as np
import pytest

import functions as fns

pytestmark = pytest.mark.gpu


def _torch_twin(fh, kind):
    """The seeded function of ``fns`` as a torch function of device tensors."""
    import torch

    if kind == "leja":
        W = torch.as_tensor(fh.W, device="cuda")
        fd = lambda X: 1.0 / (1.0 + X @ W.T)
    else:
        A = torch.as_tensor(fh.A, device="cuda")
        fd = lambda X: torch.exp(-(X @ A.T))
    fd.on_device = True
    return fd


@pytest.mark.parametrize("kind,d,t,d_out", [("leja", 10, 6.5, 3), ("gh", 8, 5.0, 2), ("leja", 40, 6.0, 17)])
def test_device_f_equals_host_f(kind, d, t, d_out):
    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes

    k = np.log((2 + np.arange(d)) / np.log(2))
    gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
    fh = fns.rational_vec(d, d_out, seed=d) if kind == "leja" else fns.exponential(d, d_out, seed=d)
    fh.vectorized = True
    host = SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=t, d_out=d_out, f=fh)
    dev = SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=t, d_out=d_out, f=_torch_twin(fh, kind))
    assert dev.n_f_evals_new == host.n_f_evals_new
    np.testing.assert_array_equal(dev._plan.keep["umap"].cpu().numpy(), host._plan.keep["umap"].cpu().numpy())
    np.testing.assert_allclose(dev.nodal_values.cpu().numpy(), host.nodal_values.cpu().numpy(), rtol=1e-14, atol=0)
    x = np.random.default_rng(2).uniform(-1, 1, (500, d)) if kind == "leja" else \
        np.random.default_rng(2).normal(size=(500, d)) / np.sqrt(2)
    np.testing.assert_allclose(dev(x).cpu().numpy(), host(x).cpu().numpy(), rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(dev.integral().cpu().numpy(), host.integral().cpu().numpy(), rtol=1e-13)


def test_device_f_wrong_width_is_an_error():
    import torch

    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes

    d = 6
    f = lambda X: torch.ones(X.shape[0], 3, dtype=torch.float64, device=X.device)
    f.on_device = True
    k = np.log((2 + np.arange(d)) / np.log(2))
    with pytest.raises(ValueError):
        SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=d), k=k, t=5.0, d_out=2, f=f)
