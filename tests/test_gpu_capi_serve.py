"""Serving queue of the C ABI (``smx_serve_*``, ``csrc/serve.cu``).

Requests of blocked and per-point plans of several interpolants and batch
sizes are submitted through ctypes, flushed (explicitly, and implicitly when a
queue fills), polled to completion, and each output is compared BIT-EXACTLY
with the package's FP32 evaluation of the same request alone (every tile of a
merged launch is evaluated as alone).  Also: tickets in submission order, poll
of a queued ticket returns 0 until its flush, argument errors are reported as
SMX_ERR_ARG without touching the queue, and a flush refused on the host fails
its own tickets only.
"""
import ctypes as C
import time

import numpy as np
import pytest
import torch

import functions as fns

pytestmark = pytest.mark.gpu


def _interp(d, t, d_out, seed):
    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes

    k = np.log((2 + np.arange(d)) / np.log(2))
    f = fns.rational(d, seed=seed) if d_out == 1 else fns.rational_vec(d, d_out, seed=seed)
    return SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=d), k=k, t=t, d_out=d_out, f=f)


@pytest.fixture(scope="module")
def plans():
    """(interpolant, kind, host plan struct) for two blocked and two per-point plans."""
    from smolyax_gb300 import _capi as capi

    out = []
    for d, t, d_out, seed in [(200, 6.5, 1, 0), (60, 6.0, 1, 1), (40, 6.0, 3, 2), (1000, 7.0, 1, 3)]:
        ip = _interp(d, t, d_out, seed)
        sp = ip.spectral_plan()
        if d_out == 1 and sp.blocked is not None and d != 1000:
            out.append((ip, capi.SMX_SERVE_BLOCKED, sp.blocked))
        else:
            out.append((ip, capi.SMX_SERVE_SPECTRAL, sp.c))
    kinds = {k for _, k, _ in out}
    assert kinds == {capi.SMX_SERVE_BLOCKED, capi.SMX_SERVE_SPECTRAL}
    return out


def _alone(kind, plan, x, d_out):
    """The request evaluated alone by smx_blocked_eval / smx_spectral_eval."""
    from smolyax_gb300 import _capi as capi

    P = int(x.shape[0])
    y = torch.empty(P, d_out, dtype=torch.float32, device="cuda")
    st = capi.stream_ptr(torch.cuda.current_stream())
    if kind == capi.SMX_SERVE_BLOCKED:
        nws = capi.size("smx_blocked_eval_workspace", C.byref(plan), P)
        ws = torch.empty(max(nws, 1), dtype=torch.uint8, device="cuda")
        capi.call("smx_blocked_eval", C.byref(plan), capi.ptr(x), P, int(x.shape[1]), capi.ptr(y), capi.ptr(ws), nws,
                  st)
    else:
        capi.call("smx_spectral_eval", C.byref(plan), capi.ptr(x), P, int(x.shape[1]), capi.ptr(y), st)
    return y


def _wait(lib, srv, ticket, limit=30.0):
    t0 = time.time()
    while True:
        r = lib.smx_serve_poll(srv, ticket)
        assert r >= 0, lib.smx_last_error_string()
        if r == 1:
            return
        assert time.time() - t0 < limit, "ticket %d not done" % ticket
        time.sleep(1e-4)


@pytest.mark.parametrize("max_items,max_plans,inflight", [(64, 8, 4), (3, 2, 1)])
def test_queue_matches_single_evaluations(plans, max_items, max_plans, inflight):
    from smolyax_gb300 import _capi as capi

    lib = capi.load()
    stream = torch.cuda.Stream()
    srv = C.c_void_p()
    assert lib.smx_serve_create(max_items, max_plans, inflight, C.c_void_p(stream.cuda_stream), C.byref(srv)) == 0
    rng = np.random.default_rng(max_items)
    reqs, tickets = [], []
    try:
        for i in range(40):
            j = int(rng.integers(len(plans)))
            ip, kind, plan = plans[j]
            P = int(rng.choice([0, 1, 7, 128, 129, 700, 5000]))
            x = torch.as_tensor(rng.uniform(-1, 1, (P, ip.d_in)), device="cuda")
            y = torch.full((P, ip.d_out), np.nan, dtype=torch.float32, device="cuda")
            torch.cuda.current_stream().synchronize()
            tk = lib.smx_serve_submit(srv, kind, C.byref(plan), C.c_void_p(x.data_ptr() if P else 0), P,
                                      ip.d_in, C.c_void_p(y.data_ptr() if P else 0))
            assert tk == i, lib.smx_last_error_string()
            reqs.append((ip, kind, plan, x, y))
            tickets.append(tk)
            if i % 11 == 10:
                assert lib.smx_serve_flush(srv) == 0
        # the last request is still queued: not done before its flush
        time.sleep(0.05)
        assert lib.smx_serve_poll(srv, tickets[-1]) == 0
        assert lib.smx_serve_flush(srv) == 0
        for tk in tickets:
            _wait(lib, srv, tk)
        for ip, kind, plan, x, y in reqs:
            if x.shape[0] == 0:
                continue
            torch.testing.assert_close(y, _alone(kind, plan, x, ip.d_out), rtol=0, atol=0)
    finally:
        lib.smx_serve_destroy(srv)


def test_argument_errors(plans):
    from smolyax_gb300 import _capi as capi

    lib = capi.load()
    srv = C.c_void_p()
    assert lib.smx_serve_create(0, 1, 1, None, C.byref(srv)) == capi.SMX_ERR_ARG
    assert lib.smx_serve_create(4, 2, 1, None, C.byref(srv)) == 0
    try:
        ip, kind, plan = plans[0]
        x = torch.zeros(5, ip.d_in, dtype=torch.float64, device="cuda")
        y = torch.zeros(5, 1, dtype=torch.float32, device="cuda")
        assert lib.smx_serve_submit(srv, 7, C.byref(plan), C.c_void_p(x.data_ptr()), 5, ip.d_in,
                                    C.c_void_p(y.data_ptr())) == capi.SMX_ERR_ARG
        assert lib.smx_serve_submit(srv, kind, C.byref(plan), C.c_void_p(x.data_ptr()), 5, ip.d_in - 1,
                                    C.c_void_p(y.data_ptr())) == capi.SMX_ERR_ARG
        assert lib.smx_serve_poll(srv, 0) == capi.SMX_ERR_ARG  # no ticket issued yet
        tk = lib.smx_serve_submit(srv, kind, C.byref(plan), C.c_void_p(x.data_ptr()), 5, ip.d_in,
                                  C.c_void_p(y.data_ptr()))
        assert tk == 0
        assert lib.smx_serve_poll(srv, 0) == 0  # queued
        assert lib.smx_serve_flush(srv) == 0
        _wait(lib, srv, 0)
        torch.testing.assert_close(y, _alone(kind, plan, x, 1), rtol=0, atol=0)
    finally:
        lib.smx_serve_destroy(srv)


def test_refused_flush_fails_its_tickets(plans):
    """A flush whose launch is refused on the host (a per-point plan whose row
    does not fit in shared memory: no launch happens) returns the error, its
    tickets poll as that error, and the queue then serves new requests."""
    from smolyax_gb300 import _capi as capi

    lib = capi.load()
    ip, kind, plan = next(p for p in plans if p[1] == capi.SMX_SERVE_SPECTRAL)
    bad = type(plan).from_buffer_copy(plan)
    bad.row = 4096  # (4096 + 32) * 128 * 4 bytes of shared memory: refused by the launcher
    srv = C.c_void_p()
    assert lib.smx_serve_create(8, 4, 2, None, C.byref(srv)) == 0
    try:
        x = torch.as_tensor(np.random.default_rng(3).uniform(-1, 1, (5, ip.d_in)), device="cuda")
        y = torch.zeros(5, ip.d_out, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        args = (C.c_void_p(x.data_ptr()), 5, ip.d_in, C.c_void_p(y.data_ptr()))
        assert lib.smx_serve_submit(srv, kind, C.byref(bad), *args) == 0
        rc = lib.smx_serve_flush(srv)
        assert rc < 0
        assert lib.smx_serve_poll(srv, 0) == rc
        assert lib.smx_serve_submit(srv, kind, C.byref(plan), *args) == 1
        assert lib.smx_serve_flush(srv) == 0
        _wait(lib, srv, 1)
        assert lib.smx_serve_poll(srv, 0) == rc
        torch.testing.assert_close(y, _alone(kind, plan, x, ip.d_out), rtol=0, atol=0)
    finally:
        lib.smx_serve_destroy(srv)
