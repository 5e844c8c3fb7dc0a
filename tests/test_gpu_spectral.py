"""Mixed-precision path: orthogonal-polynomial form evaluated in FP32.

Pins: (1) the FP64 coefficients reproduce the FP64 combination sum (host
evaluation of the orthogonal form, 1e-9 relative); (2) the FP32 GPU values
against the extended-precision values of the same data, or against the FP64
path, at 1e-6; (3) interpolation of polynomials in the index set stays exact
to FP32 accuracy.

Norms (bound 1e-6 in every case, printed per test):
* element-wise relative error, max_(p,o) |y32 - y64| / |y64| -- the Leja
  configurations and the per-point evaluator's Gauss-Hermite configurations;
* per-point norm-wise, max_p max_o |y32 - y64| / max_o |y64| -- the
  tensor-core Gauss-Hermite configurations, where some outputs are much smaller
  than the terms c_m phi_m(x) they are the sum of (condition numbers
  sum_m |c_m phi_m(x)| / |y| up to ~100 at N(0, I) points): FP32 arithmetic,
  whose rounding is relative to those terms, cannot give them 1e-6 element-wise
  accuracy.  For these the element-wise error is printed, and every element is
  also checked against 1e-6 * sum_m |c_m phi_m(x)| (error relative to the size
  of what is summed).
"""
import numpy as np
import pytest

import functions as fns
import golden_io as gio
from gpu_helpers import product_generator, rel_err

pytestmark = pytest.mark.gpu

EXACT = gio.load("exact_configs.npz")
INTERP = gio.load("interp_small.npz")


def _interp(**kw):
    from smolyax_gb300 import SmolyakBarycentricInterpolator

    return SmolyakBarycentricInterpolator(**kw)


def _phi(fam, z, n):
    out = [np.ones_like(z)]
    pm1, p = np.zeros_like(z), np.ones_like(z)
    for m in range(n):
        if fam == 0:
            a, b = (2 * m + 1) / (m + 1), m / (m + 1)
        else:
            a, b = np.sqrt(2 / (m + 1)), np.sqrt(m / (m + 1))
        pm1, p = p, a * z * p - b * pm1
        out.append(p)
    return out


def host_basis_products(ip, x):
    """[P, n_lambda] table of prod_j phi_{m_j}(z_j) over the index set (FP64,
    host), in the order of the plan's coefficient rows."""
    sp = ip.spectral_plan()
    tree = ip._tree
    tuples = tree.host_tuples(np.arange(tree.size))
    fam = sp.fam.cpu().numpy()
    a, b = sp.fa64.cpu().numpy(), sp.fb64.cpu().numpy()
    z = x * a + b
    maxdeg = ip._maxdeg
    phis = {j: _phi(fam[j], z[:, j], int(maxdeg[j])) for j in range(x.shape[1]) if maxdeg[j] > 0}
    out = np.ones((x.shape[0], len(tuples)))
    for e, nu in enumerate(tuples):
        for dd, g in nu:
            out[:, e] *= phis[dd][g]
    return out


def host_orthogonal_eval(ip, x):
    return host_basis_products(ip, x) @ ip.spectral_plan().C64.cpu().numpy()


def fp32_errors(y32, y64):
    """(element-wise max relative, per-point norm-wise max relative) errors."""
    y32, y64 = np.asarray(y32, dtype=float), np.asarray(y64, dtype=float)
    ew = float(np.max(np.abs(y32 - y64) / np.abs(y64)))
    pn = float(np.max(np.max(np.abs(y32 - y64), axis=1) / np.max(np.abs(y64), axis=1)))
    return ew, pn


def term_relative_error(ip, x, y32, y64):
    """max over elements of |y32 - y64| / sum_m |c_m phi_m(x)|."""
    S = np.abs(host_basis_products(ip, x)) @ np.abs(ip.spectral_plan().C64.cpu().numpy())
    return float(np.max(np.abs(np.asarray(y32, dtype=float) - y64) / S))


@pytest.mark.parametrize("name", [str(n) for n in INTERP["names"]][:8])
def test_small_cases_fp32(name):
    z = INTERP
    spec, k, t, d_out, f = gio.small_case(z, name)
    ip = _interp(node_gen=product_generator(spec, len(k)), k=k, t=t, d_out=d_out, f=f)
    x = z[name + "/x"]
    y64 = ip(x).cpu().numpy()
    np.testing.assert_allclose(host_orthogonal_eval(ip, x), y64, rtol=1e-9, atol=1e-10)
    y32 = ip(x, precision="fp32").cpu().numpy()
    assert y32.dtype == np.float32
    scale = max(1.0, float(np.max(np.abs(y64))))
    assert float(np.max(np.abs(y32 - y64))) / scale < 2e-6


CASES = {
    # tag: (d, t, kind, d_out, f, x); element-wise bound 1e-6 for all
    "cfg1": (10, 8.831421, "leja", 1, fns.rational(10, seed=0), np.random.default_rng(1).uniform(-1, 1, (10000, 10))),
    "cfg2": (1000, 8.224520, "leja", 1, fns.rational(1000, seed=0),
             np.random.default_rng(1).uniform(-1, 1, (256, 1000))),
    # d_out = 64: tensor-core contraction (3xTF32, FP32 accumulation in tensor memory)
    "cfg4": (200, 7.853604, "leja", 64, fns.rational_vec(200, 64, seed=0),
             np.random.default_rng(1).uniform(-1, 1, (64, 200))),
    # d_out = 8: per-point evaluator
    "cfg3alt": (100, 7.723434, "gh", 8, fns.exponential(100, 8, seed=0),
                np.random.default_rng(1).normal(size=(32, 100))),
    "cfg3": (100, 9.464636, "gh", 8, fns.exponential(100, 8, seed=0), np.random.default_rng(1).normal(size=(32, 100))),
}


@pytest.mark.parametrize("tag", list(CASES))
def test_fp32_error_bound(tag):
    """Element-wise relative error <= 1e-6 against the extended-precision values."""
    from smolyax_gb300 import nodes

    d, t, kind, d_out, f, x = CASES[tag]
    k = np.log((2 + np.arange(d)) / np.log(2))
    gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
    ip = _interp(node_gen=gen, k=k, t=t, d_out=d_out, f=f)
    y32 = ip(x, precision="fp32").cpu().numpy().astype(float)
    exact = EXACT[tag + "/y"]
    err = rel_err(y32, exact)
    print("%s: FP32 element-wise max relative error vs FP64 exact %.3e (bound 1e-06)" % (tag, err))
    assert err < 1e-6
    if x.shape[0] <= 256:
        np.testing.assert_allclose(host_orthogonal_eval(ip, x[:16]), exact[:16], rtol=1e-9)


@pytest.mark.parametrize("points", [256, 1000])
def test_fp32_leja_d200_dout64_tensor_core(points):
    """Leja d_in=200, d_out=64, |Lambda|=5000 (t=7.853604) on the tensor-core
    path: element-wise relative error <= 1e-6 against the FP64 path."""
    from smolyax_gb300 import nodes

    d = 200
    k = np.log((2 + np.arange(d)) / np.log(2))
    f = fns.rational_vec(d, 64, seed=0)
    f.vectorized = True
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=7.853604, d_out=64, f=f)
    assert ip.spectral_plan().tc is not None
    x = np.random.default_rng(11).uniform(-1, 1, (points, d))
    ew, pn = fp32_errors(ip(x, precision="fp32").cpu().numpy(), ip(x).cpu().numpy())
    print("Leja d=200 d_out=64 (%d points): element-wise %.3e, per-point norm-wise %.3e (bound 1e-06 element-wise)"
          % (points, ew, pn))
    assert ew < 1e-6


def test_forward_k_split_batch_independent():
    """Forward contraction split along K: with a 0.125 GB memory limit a panel
    chunk holds 3328 points (26 tiles for 152 SMs), so the plan contracts in
    K slices.  Element-wise error <= 1e-6 against the FP64 path, and every
    point's value bit-equal in any batch (the slice count is a constant of the
    plan; the rows checked straddle a chunk boundary in the large batch)."""
    from smolyax_gb300 import nodes

    d = 200
    k = np.log((2 + np.arange(d)) / np.log(2))
    f = fns.rational_vec(d, 64, seed=0)
    f.vectorized = True
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=7.853604, d_out=64, f=f, memory_limit=0.125)
    sp = ip.spectral_plan()
    assert sp.tc is not None and sp.tc_splits() > 1
    x = np.random.default_rng(12).uniform(-1, 1, (7000, d))
    y = ip(x, precision="fp32").cpu().numpy()
    step = sp._tc_step(len(x))
    lo, hi = step - 28, step + 72
    np.testing.assert_array_equal(y[lo:hi], ip(x[lo:hi], precision="fp32").cpu().numpy())
    ew, pn = fp32_errors(y[:512], ip(x[:512]).cpu().numpy())
    print("Leja d=200 d_out=64, %d K slices: element-wise %.3e, per-point norm-wise %.3e (bound 1e-06 element-wise)"
          % (sp.tc_splits(), ew, pn))
    assert ew < 1e-6


def test_fp32_gauss_hermite_d100_dout2048_tensor_core():
    """Gauss-Hermite d_in=100, d_out=2048, |Lambda|=20010 (t=9.464636, 159540
    nodes), 256 points ~ N(0, I): the tcgen05 3xTF32 path against the FP64
    path.  Per-point norm-wise error <= 1e-6; every element within 1e-6 of
    sum_m |c_m phi_m(x)|; element-wise error printed."""
    from smolyax_gb300 import nodes

    d, d_out = 100, 2048
    k = np.log((2 + np.arange(d)) / np.log(2))
    f = fns.exponential(d, d_out, seed=0)
    f.vectorized = True
    ip = _interp(node_gen=nodes.GaussHermite(dim=d), k=k, t=9.464636, d_out=d_out, f=f, memory_limit=8.0)
    assert ip.n_f_evals == 159540 and ip.spectral_plan().tc is not None
    x = np.random.default_rng(1).normal(size=(256, d))
    y64 = ip(x).cpu().numpy()
    y32 = ip(x, precision="fp32").cpu().numpy()
    ew, pn = fp32_errors(y32, y64)
    tr = term_relative_error(ip, x, y32, y64)
    print("GH d=100 d_out=2048: per-point norm-wise %.3e (bound 1e-06), relative to sum|terms| %.3e (bound 1e-06), "
          "element-wise %.3e" % (pn, tr, ew))
    assert pn < 1e-6 and tr < 1e-6


@pytest.mark.parametrize("t,d_out", [(7.723434, 32), (7.723434, 300)])
def test_tensor_core_path_gauss_hermite(t, d_out):
    """Gauss-Hermite, d_in = 100, vector output: the tcgen05 path against our
    FP64 path.  Per-point norm-wise error <= 1e-6 and every element within
    1e-6 of sum_m |c_m phi_m(x)|; element-wise error printed."""
    from smolyax_gb300 import nodes

    d = 100
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.GaussHermite(dim=d), k=k, t=t, d_out=d_out, f=fns.exponential(d, d_out, seed=0))
    x = np.random.default_rng(3).normal(size=(300, d))
    assert ip.spectral_plan().tc is not None
    y64 = ip(x).cpu().numpy()
    y32 = ip(x, precision="fp32").cpu().numpy().astype(float)
    ew, pn = fp32_errors(y32, y64)
    tr = term_relative_error(ip, x, y32, y64)
    print("GH d_out=%d: tensor-core FP32 per-point norm-wise %.3e, relative to sum|terms| %.3e, element-wise %.3e"
          % (d_out, pn, tr, ew))
    assert pn < 1e-6 and tr < 1e-6


def test_bf16x3_contraction_gauss_hermite():
    """precision="bf16x3": panel and coefficients split to BF16 hi/lo, three
    BF16 products per entry accumulated in FP32.  Stated accuracy: 1e-4 per-point
    norm-wise (the split keeps ~16 bits); the TF32 split (22 bits) is the
    default FP32 form."""
    from smolyax_gb300 import nodes

    d, d_out = 100, 32
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.GaussHermite(dim=d), k=k, t=7.723434, d_out=d_out,
                 f=fns.exponential(d, d_out, seed=0))
    x = np.random.default_rng(3).normal(size=(1000, d))
    assert ip.spectral_plan().tc is not None
    y64 = ip(x).cpu().numpy()
    y16 = ip(x, precision="bf16x3").cpu().numpy().astype(float)
    err = float(np.max(np.max(np.abs(y16 - y64), axis=1) / np.max(np.abs(y64), axis=1)))
    print("GH d_out=%d: bf16x3 per-point norm-wise error vs FP64 %.3e" % (d_out, err))
    assert err < 1e-4


def test_bf16x3_needs_tensor_core_form():
    from smolyax_gb300 import nodes

    d = 10
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=5.0, d_out=1, f=fns.rational(d, seed=0))
    with pytest.raises(ValueError):
        ip(np.zeros((4, d)), precision="bf16x3")


@pytest.mark.parametrize("d_out", [1, 3])
def test_host_input_overlap_equals_device_input(d_out):
    """Large host inputs are copied and evaluated in overlapped chunks: same
    values as evaluating the device copy in one call (pinned, pageable, numpy)."""
    import torch

    from smolyax_gb300 import nodes
    from smolyax_gb300.interpolation import _OVERLAP_MIN_ROWS

    d, t = 30, 6.0
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=t, d_out=d_out, f=fns.rational_vec(d, d_out, seed=4))
    x = np.random.default_rng(5).uniform(-1, 1, (2 * _OVERLAP_MIN_ROWS + 77, d))
    ref = ip(torch.as_tensor(x, device="cuda"), precision="fp32").cpu().numpy()
    for xin in (torch.from_numpy(x).pin_memory(), torch.from_numpy(x), x):
        got = ip(xin, precision="fp32")
        assert got.device.type == "cuda" and got.shape == (x.shape[0], d_out)
        # chunks may change how the last round of tiles is split: FP32 rounding only
        np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=2e-6, atol=1e-7 * np.abs(ref).max())


def test_blocked_last_round_split():
    """Tiles of a partial last round are shared by several blocks (partial sums
    added in a fixed order): same values as unsplit evaluations of the same
    points to FP32 rounding, and within the FP32 bound of the FP64 values."""
    import torch

    from smolyax_gb300 import nodes

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    d, t = 40, 6.5
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=t, d_out=1, f=fns.rational_vec(d, 1, seed=9))
    sp = ip.spectral_plan()
    assert sp.blocked is not None
    P = 128 * (sms + sms // 4) + 37  # one full round, then sms // 4 + 1 tiles for ~3 blocks each
    x = torch.as_tensor(np.random.default_rng(8).uniform(-1, 1, (P, d)), device="cuda")
    y = torch.empty(P, 1, dtype=torch.float32, device="cuda")
    sp.evaluate(x, y)
    half = 128 * (sms // 2)
    parts = []
    for a, b in ((0, half), (half, 2 * half), (2 * half, P)):
        yy = torch.empty(b - a, 1, dtype=torch.float32, device="cuda")
        sp.evaluate(x[a:b].contiguous(), yy)
        parts.append(yy)
    y_unsplit = torch.cat(parts).double()
    y64 = ip(x, precision="fp64")
    scale = y64.abs().max().item()
    assert (y.double() - y_unsplit).abs().max().item() <= 2e-6 * scale
    assert (y.double() - y64).abs().max().item() <= 1e-6 * scale


@pytest.mark.parametrize("kind,d,t", [("gh", 30, 6.5), ("leja", 30, 7.5), ("gh", 30, 7.5), ("leja", 60, 7.0)])
def test_blocked_evaluator_generic_groups(kind, d, t):
    """One-output plans on the blocked evaluator: Gauss-Hermite families, cold
    groups with non-contiguous dimensions and degree-2 cold slots (the generic
    group path) -- FP32 values within 1e-6 of the FP64 path (relative to the
    largest value)."""
    import torch

    from smolyax_gb300 import nodes

    k = np.log((2 + np.arange(d)) / np.log(2))
    gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
    f = fns.rational_vec(d, 1, seed=d) if kind == "leja" else fns.exponential(d, 1, seed=d)
    ip = _interp(node_gen=gen, k=k, t=t, d_out=1, f=f)
    sp = ip.spectral_plan()
    assert sp.blocked is not None
    rng = np.random.default_rng(d)
    x = rng.uniform(-1, 1, (3000, d)) if kind == "leja" else rng.normal(size=(3000, d)) / np.sqrt(2)
    x = torch.as_tensor(x, device="cuda")
    y32 = ip(x, precision="fp32").double()
    y64 = ip(x, precision="fp64")
    err = ((y32 - y64).abs().max() / y64.abs().max()).item()
    print("%s d=%d t=%.1f: FP32 error %.2e" % (kind, d, t, err))
    assert err < 1e-6


@pytest.mark.parametrize("bf16", [False, True])
def test_panel_segments_equal_single_walk(bf16):
    """The tape split into segments at depth-1 entries (one block of points per
    segment) writes the same panel, bit for bit, as one walk of the whole tape."""
    import torch

    from smolyax_gb300 import _capi, nodes

    d, d_out = 100, 32
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.GaussHermite(dim=d), k=k, t=7.723434, d_out=d_out,
                 f=fns.exponential(d, d_out, seed=0))
    sp = ip.spectral_plan()
    tc, kk = sp.tc, sp.keep
    assert tc is not None
    P = 300
    x = torch.as_tensor(np.random.default_rng(6).normal(size=(P, d)), device="cuda")
    K = tc["K"]
    ld = (K + 7) // 8 * 8
    dt = torch.bfloat16 if bf16 else torch.float32
    name = "smx_spectral_panel_bf16" if bf16 else "smx_spectral_panel_tf32"
    lvl1 = set(tc["lvl1"].tolist())
    st = _capi.stream_ptr(torch.cuda.current_stream())
    nws = _capi.size("smx_spectral_panel_workspace", tc["n_slots"], P)
    ws = torch.empty(max(nws, 1), dtype=torch.uint8, device="cuda")
    outs = []
    for n in (None, 2, 7, 32):
        if n is None:
            seg, n_seg = None, 1
        else:
            b = sorted(set([0, K] + [int(tc["lvl1"][min(len(lvl1) - 1, i * len(lvl1) // n)]) for i in range(1, n)]))
            assert all(v in lvl1 for v in b[:-1])
            seg, n_seg = torch.as_tensor(np.array(b, np.int32), device="cuda"), len(b) - 1
        Ah = torch.full((P, ld), 7, dtype=dt, device="cuda")
        Al = torch.full_like(Ah, 7)
        _capi.call(name, int(tc["dims"].numel()), _capi.ptr(tc["dims"]), _capi.ptr(tc["dmax"]), _capi.ptr(tc["dsoff"]),
                   tc["n_slots"], _capi.ptr(tc["tape"]), K, _capi.ptr(seg), n_seg, _capi.ptr(kk["fam_a"]),
                   _capi.ptr(kk["fam_b"]), _capi.ptr(kk["fam"]), _capi.ptr(x), P, d, _capi.ptr(Ah), _capi.ptr(Al), ld,
                   _capi.ptr(ws), nws, st)
        outs.append((Ah[:, :K].clone(), Al[:, :K].clone()))
    for Ah, Al in outs[1:]:
        assert torch.equal(Ah, outs[0][0]) and torch.equal(Al, outs[0][1])
    # the segments the plan picks for a launch start at depth-1 entries
    seg, n_seg = sp._segments(P)
    if seg is not None:
        assert all(int(v) in lvl1 for v in seg.cpu().numpy()[:-1]) and int(seg[-1]) == K


def test_blocked_tables_in_shared_memory_equal_global_tables():
    """The blocked evaluator's per-block shared-memory copy of its tables gives
    the same values, bit for bit, as reading the tables from global memory
    (the path of plans whose tables do not fit beside the tile arrays)."""
    import ctypes

    import torch

    from smolyax_gb300 import _capi, nodes

    d, t = 60, 7.0
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=t, d_out=1, f=fns.rational_vec(d, 1, seed=11))
    sp = ip.spectral_plan()
    b = sp.blocked
    assert b is not None and b.n_ent > 0 and b.n_w > 0
    P = 5000
    x = torch.as_tensor(np.random.default_rng(12).uniform(-1, 1, (P, d)), device="cuda")
    st = _capi.stream_ptr(torch.cuda.current_stream())
    nws = _capi.size("smx_blocked_eval_workspace", ctypes.byref(b), P)
    ws = torch.empty(max(nws, 1), dtype=torch.uint8, device="cuda")
    out = []
    n_ent = b.n_ent
    try:
        for ne in (n_ent, 0):  # n_ent = 0: sizes not given, tables read from global memory
            b.n_ent = ne
            y = torch.empty(P, 1, dtype=torch.float32, device="cuda")
            _capi.call("smx_blocked_eval", ctypes.byref(b), _capi.ptr(x), P, d, _capi.ptr(y), _capi.ptr(ws), nws, st)
            out.append(y)
    finally:
        b.n_ent = n_ent
    assert torch.equal(out[0], out[1])
    y64 = ip(x, precision="fp64")
    assert (out[0].double() - y64).abs().max().item() <= 1e-6 * y64.abs().max().item()


@pytest.mark.parametrize("P", [1, 130, 128 * 9 + 37, 128 * 70])
def test_blocked_small_batches_one_block_per_tile(P):
    """Launches with fewer tiles than SMs give every tile to one block, with or
    without the split workspace (their values must equal the batch kernel's,
    which never splits), within the FP32 bound of the FP64 values."""
    import ctypes

    import torch

    from smolyax_gb300 import _capi, nodes

    d, t = 40, 6.5
    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=t, d_out=1, f=fns.rational_vec(d, 1, seed=13))
    sp = ip.spectral_plan()
    b = sp.blocked
    assert b is not None
    x = torch.as_tensor(np.random.default_rng(14).uniform(-1, 1, (P, d)), device="cuda")
    st = _capi.stream_ptr(torch.cuda.current_stream())
    nws = _capi.size("smx_blocked_eval_workspace", ctypes.byref(b), P)
    ws = torch.empty(nws, dtype=torch.uint8, device="cuda")
    y_split = torch.empty(P, 1, dtype=torch.float32, device="cuda")
    y_one = torch.empty(P, 1, dtype=torch.float32, device="cuda")
    _capi.call("smx_blocked_eval", ctypes.byref(b), _capi.ptr(x), P, d, _capi.ptr(y_split), _capi.ptr(ws), nws, st)
    _capi.call("smx_blocked_eval", ctypes.byref(b), _capi.ptr(x), P, d, _capi.ptr(y_one), None, 0, st)
    y64 = ip(x, precision="fp64")
    scale = y64.abs().max().item()
    assert torch.equal(y_split, y_one)
    assert (y_split.double() - y64).abs().max().item() <= 1e-6 * scale


@pytest.mark.parametrize("d", [31, 40])
def test_blocked_row_pitch_and_alignment(d):
    """x rows with any pitch and 8-byte alignment: the evaluator's 32-byte,
    16-byte and scalar load paths give the same values, bit for bit."""
    import ctypes

    import torch

    from smolyax_gb300 import _capi, nodes

    k = np.log((2 + np.arange(d)) / np.log(2))
    ip = _interp(node_gen=nodes.Leja(dim=d), k=k, t=6.0, d_out=1, f=fns.rational_vec(d, 1, seed=15))
    sp = ip.spectral_plan()
    b = sp.blocked
    assert b is not None
    P = 128 * 5 + 3
    x0 = np.random.default_rng(16).uniform(-1, 1, (P, d))
    st = _capi.stream_ptr(torch.cuda.current_stream())
    outs = []
    # (row pitch, first column): pitch % 4 == 0 and 32-byte rows (32-byte loads),
    # 16-byte rows (16-byte loads), odd pitch or 8-byte offset (scalar loads)
    for cols, c0 in ((d, 0), (44, 0), (44, 2), (42, 0), (43, 0), (44, 1)):
        buf = np.zeros((P, cols))
        buf[:, c0:c0 + d] = x0
        xb = torch.as_tensor(buf, device="cuda")
        y = torch.empty(P, 1, dtype=torch.float32, device="cuda")
        _capi.call("smx_blocked_eval", ctypes.byref(b), ctypes.c_void_p(xb.data_ptr() + 8 * c0), P, cols,
                   _capi.ptr(y), None, 0, st)
        outs.append(y)
    for y in outs[1:]:
        assert torch.equal(outs[0], y)
    y64 = ip(torch.as_tensor(x0, device="cuda"), precision="fp64")
    assert (outs[0].double() - y64).abs().max().item() <= 1e-6 * y64.abs().max().item()


def test_fp32_and_bf16x3_input_edge_cases():
    """Empty and 1-D inputs and a wrong width on the mixed-precision paths, as
    the reference's __call__ handles them (interpolation.py:253-262)."""
    from smolyax_gb300 import nodes

    d = 10
    k = np.log((2 + np.arange(d)) / np.log(2))
    one = _interp(node_gen=nodes.Leja(dim=d), k=k, t=5.0, d_out=1, f=fns.rational(d, seed=0))
    many = _interp(node_gen=nodes.GaussHermite(dim=d), k=k, t=5.0, d_out=20, f=fns.exponential(d, 20, seed=0))
    for ip, precs in ((one, ("fp32",)), (many, ("fp32", "bf16x3"))):
        for prec in precs:
            y0 = ip(np.zeros((0, d)), precision=prec)
            assert tuple(y0.shape) == (0, ip.d_out)
            x1 = np.random.default_rng(17).normal(size=d) * 0.5
            y1 = ip(x1, precision=prec)
            assert tuple(y1.shape) == (1, ip.d_out)
            y64 = ip(x1[None, :]).cpu().numpy()
            tol = 1e-4 if prec == "bf16x3" else 2e-6
            assert np.max(np.abs(y1.cpu().numpy() - y64)) <= tol * max(1.0, np.max(np.abs(y64)))
            with pytest.raises(AssertionError):
                ip(np.zeros((3, d + 1)), precision=prec)
