"""Allocation-free FP64 evaluation (``smx_eval_f64_noalloc``), through the C ABI.

Some callers cannot allocate device memory while they evaluate: foreign-
language hosts without a CUDA allocator, services whose device memory is owned
by a pool, code that must not call cudaMalloc because it synchronises the
device.  The entry point gives them the FP64 evaluation with a library-owned
scratch array; its results must equal those of the workspace-taking
``smx_eval`` (same kernels, same arithmetic) on consecutive calls.

This file is collected last on purpose; it builds its own interpolant so that
it also passes alone in a fresh process.
"""
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_scratch_bytes():
    """SMX_STATIC_SCRATCH_BYTES as the public header defines it."""
    hdr = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include", "smolyax_gb300.h")
    m = re.search(r"#define\s+SMX_STATIC_SCRATCH_BYTES\s+\((\d+)u\s*<<\s*(\d+)\)", open(hdr).read())
    assert m, "SMX_STATIC_SCRATCH_BYTES not found in the header"
    return int(m.group(1)) << int(m.group(2))


def test_noalloc_matches_workspace_entry_point():
    import torch

    from smolyax_gb300 import SmolyakBarycentricInterpolator, _capi, nodes

    lib = _capi.load()
    d = 10
    k = np.log((2 + np.arange(d)) / np.log(2))
    rng = np.random.default_rng(7)
    w = rng.uniform(0, 1, d) / (np.arange(d) + 1) ** 2
    f = lambda x: np.array([1.0 / (1.0 + 0.5 * np.dot(w, x) / w.sum()), np.cos(x[0]) * x[1]])
    ip = SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=d), k=k, t=8.831421, d_out=2, f=f)
    plan = ip._plan
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = _capi.stream_ptr(torch.cuda.current_stream())
    P = 4096
    for call in range(2):  # two calls in a row; the second must not see the first's scratch
        x = torch.as_tensor(rng.uniform(-1, 1, (P, d)), device=dev)
        y_ws = torch.empty(P, 2, dtype=torch.float64, device=dev)
        y_na = torch.full((P, 2), float("nan"), dtype=torch.float64, device=dev)
        ws = torch.empty(_capi.size("smx_eval_workspace", plan.ref(), P, 64), dtype=torch.uint8, device=dev)
        _capi.call("smx_eval", plan.ref(), 64, _capi.ptr(x), P, d, _capi.ptr(y_ws), _capi.ptr(ws), ws.numel(), stream)
        _capi.call("smx_eval_f64_noalloc", plan.ref(), _capi.ptr(x), P, d, _capi.ptr(y_na), stream)
        torch.cuda.synchronize()
        np.testing.assert_allclose(y_na.cpu().numpy(), y_ws.cpu().numpy(), rtol=1e-12, atol=0.0)
    # the largest batch that fits the static scratch is evaluated like smx_eval
    most = _static_scratch_bytes() // (8 * plan.c.n_values)
    x = torch.as_tensor(rng.uniform(-1, 1, (most + 1, d)), device=dev)
    y_ws = torch.empty(most, 2, dtype=torch.float64, device=dev)
    y_na = torch.full((most + 1, 2), float("nan"), dtype=torch.float64, device=dev)
    ws = torch.empty(_capi.size("smx_eval_workspace", plan.ref(), most, 64), dtype=torch.uint8, device=dev)
    _capi.call("smx_eval", plan.ref(), 64, _capi.ptr(x), most, d, _capi.ptr(y_ws), _capi.ptr(ws), ws.numel(), stream)
    _capi.call("smx_eval_f64_noalloc", plan.ref(), _capi.ptr(x), most, d, _capi.ptr(y_na), stream)
    torch.cuda.synchronize()
    np.testing.assert_allclose(y_na[:most].cpu().numpy(), y_ws.cpu().numpy(), rtol=1e-12, atol=0.0)
    # one point more is rejected before any launch, and the message names the limit
    rc = lib.smx_eval_f64_noalloc(plan.ref(), _capi.ptr(x), most + 1, d, _capi.ptr(y_na), stream)
    assert rc == -2
    msg = lib.smx_last_error_string().decode()
    assert "static scratch" in msg and ("at most %d points" % most) in msg
    assert bool(torch.isnan(y_na[most]).all())
