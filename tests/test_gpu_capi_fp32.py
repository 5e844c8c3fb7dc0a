"""The FP32 form and its VJP through the C ABI alone: ``smx_fp32_plan_create``
on an FP64 plan and its index-set tree, ``smx_eval(plan, 32, ...)``,
``smx_fp32_eval`` and ``smx_vjp``, for each of the three FP32 evaluators.
The library builds the same FP64 coefficients as the Python package (the
scatter into the index set sums each entry's rows in row order: the same on
every call), checked bit for bit, and the same tables; its launch choices
(segments of the per-point and panel kernels, split-K slices) follow its own
rules, so the values, dL/dx and dL/d(rows of F64) are compared with the
package's at FP32 rounding (2^-20 of their scale), the two C entry points
with each other bit for bit, and the values with the FP64 path at the 1e-6
bound (element-wise: Leja cases).  The handle also carries the FP64 tables
of the orthogonal form: ``smx_eval(plan, 64, ...)`` then equals the
package's precision "fp64" bit for bit."""
import ctypes

import numpy as np
import pytest

import functions as fns

pytestmark = pytest.mark.gpu


def _fp32_plan(ip):
    import torch

    from smolyax_gb300 import _capi

    lib = _capi.load()
    tree = ip._tree
    t = _capi.SmxTree(tree.size, tree.parent.data_ptr(), tree.dim.data_ptr(), tree.deg.data_ptr(),
                      tree.rem.data_ptr(), tree.first_child.data_ptr(), tree.n_child.data_ptr())
    sp = ip.spectral_plan()
    fam = np.ascontiguousarray(sp.fam.cpu().numpy(), dtype=np.int32)
    fa = np.ascontiguousarray(sp.fa64.cpu().numpy())
    fb = np.ascontiguousarray(sp.fb64.cpu().numpy())
    h = ctypes.c_void_p()
    rc = lib.smx_fp32_plan_create(ip._plan.ref(), ctypes.byref(t), fam.ctypes.data, fa.ctypes.data, fb.ctypes.data,
                                  8.0, ctypes.byref(h), _capi.stream_ptr(torch.cuda.current_stream()))
    assert rc == 0, lib.smx_last_error_string()
    return lib, h


@pytest.mark.parametrize("kind,d,t,d_out,evaluator", [("leja", 40, 6.5, 1, 0), ("gh", 12, 6.0, 3, 1),
                                                      ("leja", 30, 6.0, 20, 2), ("leja", 1000, 8.22452, 1, 0)])
def test_fp32_form_and_vjp_through_the_c_abi(kind, d, t, d_out, evaluator):
    import torch

    from smolyax_gb300 import SmolyakBarycentricInterpolator, _capi, nodes

    k = np.log((2 + np.arange(d)) / np.log(2))
    gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
    f = fns.rational_vec(d, d_out, seed=d) if kind == "leja" else fns.exponential(d, d_out, seed=d)
    f.vectorized = True
    ip = SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=t, d_out=d_out, f=f)
    lib, h = _fp32_plan(ip)
    try:
        ev, nl, coef = ctypes.c_int(), ctypes.c_int64(), ctypes.c_void_p()
        assert lib.smx_fp32_plan_info(h, ctypes.byref(ev), ctypes.byref(nl), ctypes.byref(coef)) == 0
        assert ev.value == evaluator and nl.value == ip._tree.size
        sp = ip.spectral_plan()

        class _Dev:  # the library's device array of coefficients, viewed through the CUDA array interface
            __cuda_array_interface__ = {"shape": (nl.value, d_out), "typestr": "<f8", "data": (coef.value, False),
                                        "version": 3}

        torch.cuda.synchronize()
        assert torch.equal(torch.as_tensor(_Dev(), device="cuda"), sp.C64)
        st = _capi.stream_ptr(torch.cuda.current_stream())
        rng = np.random.default_rng(3)
        P = 777
        x = torch.as_tensor(rng.uniform(-1, 1, (P, d)) if kind == "leja" else rng.normal(size=(P, d)) / np.sqrt(2),
                            device="cuda")
        # evaluation through smx_eval(plan, 32, ...) with plan->fp32 set, and through smx_fp32_eval
        ip._plan.c.fp32 = h
        try:
            nws = lib.smx_eval_workspace(ip._plan.ref(), P, 32)
            ws = torch.empty(max(nws, 1), dtype=torch.uint8, device="cuda")
            y1 = torch.full((P, d_out), float("nan"), dtype=torch.float32, device="cuda")
            _capi.call("smx_eval", ip._plan.ref(), 32, _capi.ptr(x), P, d, _capi.ptr(y1), _capi.ptr(ws), nws, st)
        finally:
            ip._plan.c.fp32 = None
        y2 = torch.full((P, d_out), float("nan"), dtype=torch.float32, device="cuda")
        nws = lib.smx_fp32_workspace(h, P)
        ws = torch.empty(max(nws, 1), dtype=torch.uint8, device="cuda")
        _capi.call("smx_fp32_eval", h, _capi.ptr(x), P, d, _capi.ptr(y2), _capi.ptr(ws), nws, st)
        assert lib.smx_fp32_plan_check(h, st) == 0
        ref = ip(x, precision="fp32")
        y64 = ip(x, precision="fp64")
        torch.cuda.synchronize()
        assert torch.equal(y1, y2)
        dy = float((y1 - ref).abs().max())
        assert dy <= 2.0**-20 * float(ref.abs().max()), dy
        if kind == "leja":
            assert float(((y1.double() - y64).abs() / y64.abs()).max()) < 1e-6
        # without the FP32 form, precision 32 is refused
        assert lib.smx_eval(ip._plan.ref(), 32, _capi.ptr(x), P, d, _capi.ptr(y1), None, 0, st) == -5
        # FP64: the handle carries the FP64 tables of the orthogonal form, and
        # smx_eval(plan, 64, ...) with plan->fp32 set evaluates through them -- the
        # same tables and kernel as the package's precision "fp64", bit for bit
        assert lib.smx_fp32_plan_has_fp64(h) == 1
        y64c = torch.full((P, d_out), float("nan"), dtype=torch.float64, device="cuda")
        ip._plan.c.fp32 = h
        try:
            nws = lib.smx_eval_workspace(ip._plan.ref(), P, 64)
            ws = torch.empty(max(nws, 1), dtype=torch.uint8, device="cuda")
            _capi.call("smx_eval", ip._plan.ref(), 64, _capi.ptr(x), P, d, _capi.ptr(y64c), _capi.ptr(ws), nws, st)
        finally:
            ip._plan.c.fp32 = None
        assert ip._fp64_orthogonal() is not None
        torch.cuda.synchronize()
        assert torch.equal(y64c, y64)
        # vector-Jacobian products
        g = torch.as_tensor(rng.normal(size=(P, d_out)).astype(np.float32), device="cuda")
        R = int(ip._plan.c.n_entries)
        dx = torch.full((P, d), float("nan"), dtype=torch.float64, device="cuda")
        dF = torch.full((R, d_out), float("nan"), dtype=torch.float64, device="cuda")
        nws = lib.smx_vjp_workspace(h, P)
        ws = torch.empty(max(nws, 1), dtype=torch.uint8, device="cuda")
        _capi.call("smx_vjp", h, _capi.ptr(x), P, d, _capi.ptr(g), d_out, _capi.ptr(dx), d, _capi.ptr(dF),
                   _capi.ptr(ws), nws, st)
        assert lib.smx_fp32_plan_check(h, st) == 0
        dx_ref, dC_ref = sp.vjp(x, g)
        dF_ref = sp.coefficient_adjoint(dC_ref)
        torch.cuda.synchronize()
        ddx = float((dx - dx_ref).abs().max())
        assert ddx <= 2.0**-20 * float(dx_ref.abs().max()), ddx
        ddF = float((dF - dF_ref).abs().max())
        assert ddF <= 2.0**-20 * float(dF_ref.abs().max()), ddF
    finally:
        lib.smx_fp32_plan_destroy(h)
