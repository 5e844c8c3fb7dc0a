"""Continuous-batching request loop over many resident interpolants.

A :class:`Server` keeps built interpolants (plans, coefficients) resident on
the device and serves evaluation and gradient requests of different
interpolants and batch sizes:

* admission -- requests wait in FIFO order and are admitted while a stream
  slot is free and their device memory (inputs, outputs, scratch) fits the
  budget; a request that can never fit is rejected;
* batching  -- at every scheduling step, the admitted FP32 evaluations whose
  plans use a CUDA-core evaluator are merged into one persistent launch per
  evaluator kind (``smx_blocked_eval_batch`` for one-output plans with blocked
  tables, ``smx_spectral_eval_batch`` for the others: blocks take 128-point
  tiles of any request from a shared counter); tensor-core evaluations, FP64
  evaluations and gradients run on their own streams, so their work overlaps
  on the device;
* completion -- each admission group records a CUDA event; the loop polls the
  events, copies results to the host, frees memory and slots, and admits
  requests that arrived meanwhile.

Results are identical to evaluating each request alone (same kernels per
128-point tile).  Gradient requests return the vector-Jacobian product
dL/dx for a cotangent (default: ones), shape [P, d_in].
"""
from __future__ import annotations

import collections
import itertools
import threading
import time

import numpy as np
import torch

from . import _capi as capi
from ._capi import call, ptr


class Request:
    """One evaluation or gradient request; ``result`` is set when done."""

    _ids = itertools.count()

    def __init__(self, name, x, op="eval", precision="fp32", cotangent=None):
        if op not in ("eval", "grad"):
            raise ValueError("op must be 'eval' or 'grad'")
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        self.id = next(self._ids)
        self.name = name
        self.op = op
        self.precision = precision
        self.x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
        if self.x.ndim == 1:
            self.x = self.x[None, :]
        self.cotangent = cotangent
        self.t_submit = None
        self.t_admit = None
        self.t_done = None
        self.result = None
        self.error = None
        self.done = threading.Event()

    @property
    def points(self):
        return int(self.x.shape[0])

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit


class _Group:
    """Requests launched together: one stream, one completion event."""

    def __init__(self, stream, reqs, nbytes):
        self.stream = stream
        self.reqs = reqs
        self.nbytes = nbytes
        self.event = torch.cuda.Event()
        self.keep = []
        self.outputs = []


class Server:
    """Request loop over resident interpolants (see the module docstring)."""

    def __init__(self, interpolants: dict, memory_budget: float = 8.0, n_streams: int = 8):
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        self.ips = dict(interpolants)
        self.names = list(self.ips)
        self.spec = {}
        for name, ip in self.ips.items():
            self.spec[name] = ip.spectral_plan()
            self.spec[name]._backward_ops()  # gradient operands built before serving starts
        self.budget = int(memory_budget * 1024**3)
        self.in_use = 0
        self.streams = [torch.cuda.Stream(device=self.dev) for _ in range(n_streams)]
        self.free_streams = collections.deque(self.streams)
        self.waiting = collections.deque()
        self.inflight = []
        self.lock = threading.Lock()
        self.completed = []
        self.rejected = []
        self.batch_launches = 0
        self.launches = 0
        self.admitted = 0

    # ------------------------------------------------------------------ interface
    def submit(self, req: Request) -> Request:
        if req.name not in self.ips:
            raise KeyError(req.name)
        if req.x.shape[1] != self.ips[req.name].d_in:
            raise ValueError("input width %d != d_in %d" % (req.x.shape[1], self.ips[req.name].d_in))
        req.t_submit = time.perf_counter()
        with self.lock:
            self.waiting.append(req)
        return req

    def idle(self):
        with self.lock:
            return not self.waiting and not self.inflight

    def step(self):
        """One scheduling step: complete finished groups, then admit and launch."""
        self._poll()
        self._admit()

    def drain(self, timeout=600.0):
        t0 = time.perf_counter()
        while not self.idle():
            self.step()
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("server did not drain")
            time.sleep(0.0002)

    # ------------------------------------------------------------------ internals
    def request_bytes(self, req):
        ip = self.ips[req.name]
        P, d_in, d_out = req.points, ip.d_in, ip.d_out
        b = P * d_in * 8 + P * d_out * (4 if req.precision == "fp32" else 8)
        sp = self.spec[req.name]
        if req.op == "grad":
            bwd = sp._bwd or {}
            K = bwd.get("ldk", ip._tree.size)
            b += P * d_in * 8 + P * K * 4 + P * 4 * ((d_out + 3) // 4 * 4) * 3 + P * 4 * bwd.get("n_slots", d_in)
        elif req.precision == "fp64":
            b += P * ip._plan.c.n_values * 8
        elif sp.tc is not None:
            b += min(P, 1 << 20) * sp.tc["ldk"] * 8
        return b

    def _kind(self, req):
        """'blocked' / 'stream': merged into a persistent multi-plan launch; None: own launch."""
        sp = self.spec[req.name]
        if req.op != "eval" or req.precision != "fp32" or sp.tc is not None:
            return None
        if sp.blocked is not None:
            # a request of a full round of tiles or more fills the GPU alone (and
            # is then evaluated exactly as alone, with the last-round split)
            return None if req.points > 128 * self.sms else "blocked"
        return "stream"

    def _admit(self):
        batches, singles = {}, []
        with self.lock:
            avail = len(self.free_streams)  # streams not yet promised in this step
            while self.waiting:
                req = self.waiting[0]
                nb = self.request_bytes(req)
                if nb > self.budget:
                    self.waiting.popleft()
                    req.error = "request needs %d bytes, more than the server's budget" % nb
                    req.t_done = time.perf_counter()
                    req.done.set()
                    self.rejected.append(req)
                    continue
                if self.in_use + nb > self.budget:
                    break
                kind = self._kind(req)
                if kind is None or kind not in batches:
                    if avail < 1:
                        break
                    avail -= 1  # an own launch, or the first request of a merged launch
                self.waiting.popleft()
                if kind is None:
                    singles.append((req, nb, self.free_streams.popleft()))
                else:
                    batches.setdefault(kind, []).append((req, nb))
                self.in_use += nb
                self.admitted += 1
            streams = {kind: self.free_streams.popleft() for kind in batches}
        now = time.perf_counter()
        for kind, batch in batches.items():
            self._launch_batch(kind, batch, streams[kind], now)
        for req, nb, stream in singles:
            try:
                self._launch_single(req, nb, stream, now)
            except (RuntimeError, ValueError) as e:  # the plan cannot serve this request
                req.error = str(e)
                req.t_done = time.perf_counter()
                req.done.set()
                with self.lock:
                    self.rejected.append(req)
                    self.in_use -= nb
                    self.free_streams.append(stream)

    def _h2d(self, req, stream):
        xh = torch.from_numpy(req.x).pin_memory()
        with torch.cuda.stream(stream):
            xd = torch.empty(req.x.shape, dtype=torch.float64, device=self.dev)
            xd.copy_(xh, non_blocking=True)
        return xh, xd

    def _launch_batch(self, kind, batch, stream, now):
        g = _Group(stream, [r for r, _ in batch], sum(nb for _, nb in batch))
        plan_idx = {}
        plans = []
        for req, _ in batch:
            if req.name not in plan_idx:
                plan_idx[req.name] = len(plans)
                sp = self.spec[req.name]
                plans.append(sp.blocked if kind == "blocked" else sp.c)
        struct = capi.SmxBlocked if kind == "blocked" else capi.SmxSpectral
        arr = (struct * len(plans))(*plans)
        items = (capi.SmxWork * len(batch))()
        with torch.cuda.stream(stream):
            for i, (req, _) in enumerate(batch):
                req.t_admit = now
                xh, xd = self._h2d(req, stream)
                y = torch.empty(req.points, self.ips[req.name].d_out, dtype=torch.float32, device=self.dev)
                g.keep += [xh, xd]
                g.outputs.append(y)
                items[i].plan = plan_idx[req.name]
                items[i].x = xd.data_ptr()
                items[i].P = req.points
                items[i].ldx = req.x.shape[1]
                items[i].y = y.data_ptr()
            if kind == "blocked":
                nws = capi.size("smx_blocked_eval_batch_workspace", len(plans), len(batch))
            else:
                max_dout = max(p.d_out for p in plans)
                nws = capi.size("smx_spectral_eval_batch_workspace", len(plans), len(batch), max_dout)
            ws = torch.empty(nws, dtype=torch.uint8, device=self.dev)
            g.keep.append(ws)
            fn = "smx_blocked_eval_batch" if kind == "blocked" else "smx_spectral_eval_batch"
            call(fn, arr, len(plans), items, len(batch), ptr(ws), ws.numel(), capi.stream_ptr(stream))
            g.host = [torch.empty(y.shape, dtype=y.dtype, pin_memory=True) for y in g.outputs]
            for h, y in zip(g.host, g.outputs):
                h.copy_(y, non_blocking=True)
            g.event.record(stream)
        self.batch_launches += 1
        self.launches += 1
        self.inflight.append(g)

    def _launch_single(self, req, nb, stream, now):
        g = _Group(stream, [req], nb)
        ip = self.ips[req.name]
        req.t_admit = now
        with torch.cuda.stream(stream):
            xh, xd = self._h2d(req, stream)
            g.keep += [xh, xd]
            if req.op == "eval":
                y = ip(xd, precision=req.precision)
            else:
                cot = req.cotangent
                cot = torch.ones(req.points, ip.d_out, dtype=torch.float32, device=self.dev) if cot is None else \
                    torch.as_tensor(np.asarray(cot), dtype=torch.float32, device=self.dev)
                y, _ = self.spec[req.name].vjp(xd, cot, need_x=True, need_coef=False, check=False)
            g.outputs.append(y)
            g.host = [torch.empty(y.shape, dtype=y.dtype, pin_memory=True)]
            g.host[0].copy_(y, non_blocking=True)
            g.event.record(stream)
        self.launches += 1
        self.inflight.append(g)

    def _poll(self):
        done = [g for g in self.inflight if g.event.query()]
        if not done:
            return
        now = time.perf_counter()
        for g in done:
            self.inflight.remove(g)
            for req, h in zip(g.reqs, g.host):
                req.result = h.numpy()
                req.t_done = now
                req.done.set()
                self.completed.append(req)
            with self.lock:
                self.in_use -= g.nbytes
                self.free_streams.append(g.stream)

    # ------------------------------------------------------------------ statistics
    def stats(self):
        lat = np.array([r.latency for r in self.completed]) if self.completed else np.zeros(1)
        evals = sum(r.points * self.ips[r.name].d_out for r in self.completed if r.op == "eval")
        return dict(
            completed=len(self.completed), rejected=len(self.rejected), launches=self.launches,
            batch_launches=self.batch_launches, p50_ms=float(np.percentile(lat, 50) * 1e3),
            p99_ms=float(np.percentile(lat, 99) * 1e3), evals=int(evals),
        )


def replay(server: Server, arrivals, requests, timeout=600.0):
    """Submit ``requests[i]`` at time ``arrivals[i]`` (seconds from start) while
    running the loop; returns the wall time until the last completion."""
    order = np.argsort(arrivals)
    t0 = time.perf_counter()
    i = 0
    while i < len(order) or not server.idle():
        now = time.perf_counter() - t0
        while i < len(order) and arrivals[order[i]] <= now:
            server.submit(requests[order[i]])
            i += 1
        server.step()
        if now > timeout:
            raise TimeoutError("replay did not finish")
        time.sleep(0.0001)
    return time.perf_counter() - t0
