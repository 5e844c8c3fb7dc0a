"""FP64 path on the GPU against the reference's outputs (golden vectors).

Both FP64 evaluators are checked: the default ("fp64": the orthogonal form in
FP64 for Leja / Gauss-Hermite plans, ``csrc/spectral64.cu``) and
the reference's combination sum ("fp64_barycentric", ``csrc/eval64.cu``).
Small cases: 1e-12 relative against the reference's values (absolute floor
1e-13, times the output scale for the orthogonal form); gradients 1e-10
relative with an absolute floor, NaN exactly where the reference has NaN.
Benchmark workloads: the contract of ``gpu_helpers.check_fp64`` -- at least as
accurate as the reference against the extended-precision value of the same
data, and within 1e-12 of it wherever the reference is.
"""
import numpy as np
import pytest

import functions as fns
import golden_io as gio
from gpu_helpers import assert_close_nan, check_fp64, check_fp64_grad, product_generator, rel_err

pytestmark = pytest.mark.gpu

INTERP = gio.load("interp_small.npz")
CFG = gio.load("interp_configs.npz")
EXACT = gio.load("exact_configs.npz")


def _interp(**kw):
    from smolyax_gb300 import SmolyakBarycentricInterpolator

    return SmolyakBarycentricInterpolator(**kw)


@pytest.mark.parametrize("precision", ["fp64", "fp64_barycentric"])
@pytest.mark.parametrize("name", [str(n) for n in INTERP["names"]])
def test_small_cases(name, precision):
    z = INTERP
    spec, k, t, d_out, f = gio.small_case(z, name)
    ip = _interp(node_gen=product_generator(spec, len(k)), k=k, t=t, d_out=d_out, f=f)
    x = z[name + "/x"]
    y = ip(x, precision=precision).cpu().numpy()
    # the absolute floor: 1e-13, times the output scale for the orthogonal form,
    # which reproduces a nodal value (here an exact 0 at a grid point) to
    # rounding instead of by the barycentric formula's one-hot
    ref = np.asarray(z[name + "/y"], dtype=float)
    floor = 1e-13 * (max(1.0, float(np.abs(ref).max())) if precision == "fp64" else 1.0)
    np.testing.assert_allclose(y, ref, rtol=1e-12, atol=floor)
    g = ip.gradient(x[:-1]).cpu().numpy()
    assert_close_nan(g, z[name + "/grad"], rtol=1e-10, atol=1e-11)
    np.testing.assert_allclose(ip.integral().cpu().numpy(), z[name + "/integral"], rtol=1e-12, atol=1e-12)
    assert (ip.n_f_evals, ip.n_f_evals_new) == tuple(int(v) for v in z[name + "/n_f_evals"])


@pytest.mark.parametrize("precision", ["fp64", "fp64_barycentric"])
def test_config1_full(precision):
    from smolyax_gb300 import nodes

    d = 10
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=8.831421, d_out=1, f=fns.rational(d, seed=0))
    x = np.random.default_rng(1).uniform(-1, 1, (10000, d))
    check_fp64(ip(x, precision=precision).cpu().numpy(), CFG["cfg1/y"], EXACT["cfg1/y"])
    check_fp64_grad(ip.gradient(x[:64]).cpu().numpy(), CFG["cfg1/grad"], EXACT["cfg1/grad"])
    check_fp64(ip.integral().cpu().numpy(), CFG["cfg1/integral"], EXACT["cfg1/integral"], what="integral")
    assert (ip.n_f_evals, ip.n_f_evals_new) == tuple(int(v) for v in CFG["cfg1/n_f_evals"])


@pytest.mark.parametrize("precision", ["fp64", "fp64_barycentric"])
def test_config2_subset(precision):
    from smolyax_gb300 import nodes

    d = 1000
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=8.224520, d_out=1, f=fns.rational(d, seed=0))
    x = np.random.default_rng(1).uniform(-1, 1, (256, d))
    np.testing.assert_allclose([x.sum(), (x * x).sum()], CFG["cfg2/x_checksum"], rtol=1e-14)
    check_fp64(ip(x, precision=precision).cpu().numpy(), CFG["cfg2/y"], EXACT["cfg2/y"])
    check_fp64_grad(ip.gradient(x[:4]).cpu().numpy(), CFG["cfg2/grad"], EXACT["cfg2/grad"])
    check_fp64(ip.integral().cpu().numpy(), CFG["cfg2/integral"], EXACT["cfg2/integral"], what="integral")
    assert (ip.n_f_evals, ip.n_f_evals_new) == tuple(int(v) for v in CFG["cfg2/n_f_evals"])


@pytest.mark.parametrize("precision", ["fp64", "fp64_barycentric"])
def test_config4_subset(precision):
    from smolyax_gb300 import nodes

    d = 200
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=7.853604, d_out=64, f=fns.rational_vec(d, 64, seed=0))
    x = np.random.default_rng(1).uniform(-1, 1, (64, d))
    check_fp64(ip(x, precision=precision).cpu().numpy(), CFG["cfg4/y"], EXACT["cfg4/y"])
    check_fp64_grad(ip.gradient(x[:3]).cpu().numpy(), CFG["cfg4/grad"], EXACT["cfg4/grad"])
    check_fp64(ip.integral().cpu().numpy(), CFG["cfg4/integral"], EXACT["cfg4/integral"], what="integral")


@pytest.mark.parametrize("precision", ["fp64", "fp64_barycentric"])
@pytest.mark.parametrize("tag,t", [("cfg3alt", 7.723434), ("cfg3", 9.464636)])
def test_config3_gauss_hermite(tag, t, precision):
    from smolyax_gb300 import nodes

    d = 100
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.GaussHermite(dim=d), k=k, t=t, d_out=8, f=fns.exponential(d, 8, seed=0))
    x = np.random.default_rng(1).normal(size=(32, d))
    check_fp64(ip(x, precision=precision).cpu().numpy(), CFG[tag + "/y"], EXACT[tag + "/y"])
    check_fp64(ip.integral().cpu().numpy(), CFG[tag + "/integral"], EXACT[tag + "/integral"], what="integral")
    assert (ip.n_f_evals, ip.n_f_evals_new) == tuple(int(v) for v in CFG[tag + "/n_f_evals"])
    if tag == "cfg3alt":
        check_fp64_grad(ip.gradient(x[:2]).cpu().numpy(), CFG[tag + "/grad"], EXACT[tag + "/grad"])


def test_f_evals_reuse_and_shapes():
    from smolyax_gb300 import nodes

    d = 3
    k = [1.0, 1.3, 2.0]
    f = lambda x: np.array([np.cos(x[0]) * x[1] + x[2] ** 2, x[0]])
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=4.0, d_out=2)
    fe = ip.set_f(f=f)
    assert ip.n_f_evals_new == ip.n_f_evals == len(fe)
    ip2 = _interp(node_gen=nodes.Leja(dim=d), k=k, t=4.0, d_out=2)
    ip2.set_f(f=f, f_evals=fe)
    assert ip2.n_f_evals_new == 0
    x = np.array([0.1, -0.2, 0.3])
    assert tuple(ip(x).shape) == (1, 2)
    assert tuple(ip(np.zeros((0, d))).shape) == (0, 2)
    np.testing.assert_array_equal(ip(x).cpu().numpy(), ip2(x).cpu().numpy())
    # non-nested cache layout: one dictionary per multi-index
    gh = _interp(node_gen=nodes.GaussHermite(dim=d), k=k, t=4.0, d_out=2)
    fe2 = gh.set_f(f=f)
    assert all(isinstance(v, dict) for v in fe2.values())
    assert sum(len(v) for v in fe2.values()) == gh.n_f_evals_new


def test_constant_only_and_chunking():
    from smolyax_gb300 import nodes

    ip = _interp(node_gen=nodes.Leja(dim=2), k=[1.0, 2.0], t=0.5, d_out=1, f=lambda x: np.array([3.0]))
    np.testing.assert_array_equal(ip(np.ones((5, 2))).cpu().numpy(), 3.0)
    np.testing.assert_array_equal(ip.gradient(np.ones((2, 2))).cpu().numpy(), 0.0)
    d = 5
    k = np.log((2 + np.arange(d)) / np.log(2))
    f = fns.rational(d, seed=3)
    a = _interp(node_gen=nodes.Leja(dim=d), k=k, t=6.0, d_out=1, f=f)
    b = _interp(node_gen=nodes.Leja(dim=d), k=k, t=6.0, d_out=1, f=f, memory_limit=1e-6)
    x = np.random.default_rng(2).uniform(-1, 1, (999, d))
    bary = "fp64_barycentric"  # the evaluator that chunks by the memory limit
    np.testing.assert_array_equal(a(x, precision=bary).cpu().numpy(), b(x, precision=bary).cpu().numpy())
    np.testing.assert_array_equal(a(x).cpu().numpy(), b(x).cpu().numpy())
    np.testing.assert_array_equal(a(x).cpu().numpy(), a(x).cpu().numpy())
