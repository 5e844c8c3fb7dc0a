"""Continuous-batching request loop over many resident interpolants.

A :class:`Server` keeps built interpolants (plans, coefficients, backward
operands) resident on the device and serves evaluation and gradient requests
of different interpolants and batch sizes:

* admission -- requests wait in FIFO order and are admitted while a stream is
  free and their device memory (inputs, outputs, the scratch of the kernels
  that will run) fits the budget; a request that can never fit the budget is
  rejected;
* batching  -- at every scheduling step the admitted requests are merged by
  kind, one launch (and one stream) per kind:

  - FP32 evaluations of one-output plans with blocked tables and of plans on
    the per-point evaluator: one persistent multi-plan launch each
    (``smx_blocked_eval_batch``, ``smx_spectral_eval_batch``: blocks take
    128-point tiles of any request from a shared counter);
  - every other request (tensor-core evaluations, FP64 evaluations, gradients)
    merges with the admitted requests of the same interpolant, operation and
    precision: their points are copied into one device array and evaluated
    (or differentiated) by one call, whose rows are then handed back per
    request.  These paths compute every point independently of the others,
    so a request's rows are the same alone and in the merged call.  (A blocked
    one-output request large enough to fill the GPU alone runs alone: its
    tiles of the last round may be shared by several blocks.)

  Launches of different kinds run on different streams, so their work
  overlaps on the device;
* priorities -- a launch whose estimated work (multiply-adds: points x
  |Lambda| x d_out, x3 for gradients) is at most ``fast_work`` runs on one of
  ``n_fast_streams`` streams of the device's highest priority, the others on
  ``n_streams`` normal streams.  The block scheduler then starts the blocks of
  a small launch as soon as blocks of a running large launch retire, instead
  of after all of the large launch's blocks, and a small request that finds
  every normal stream busy is still admitted (the scan of the FIFO queue
  passes requests whose class has no free stream);
* staging   -- inputs are copied from the request's numpy array into a pinned
  host arena allocated once (no page-locking per request; the host copies run
  on torch's intra-op threads), then to the device without blocking the host;
  results come back into the arena the same way.
  When the arena is full, a launch takes a one-off pinned buffer instead
  (counted in ``stats()["staging_spills"]``);
* completion -- each launch records a CUDA event; the loop polls the events,
  hands results to the requests, frees device memory, stream and staging
  space, and admits requests that arrived meanwhile.
* host threads -- with ``host_threads`` > 0 the preparation of a launch
  (staging copies, kernel launches) and the hand-back of its results run on a
  pool of host threads, so that the copies of a large request do not hold up
  the scheduling of the others (the copies and the CUDA calls release the
  interpreter lock); with 0 everything runs on the caller's thread.  A launch that fails
  (an error raised while it is prepared) fails its requests with the message
  and gives back everything it took.

Results are identical to evaluating each request alone.  Gradient requests
return the vector-Jacobian product dL/dx for a cotangent (default: ones),
shape [P, d_in].
"""
from __future__ import annotations

import bisect
import collections
import itertools
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from . import _capi as capi
from ._capi import call, ptr

_ALIGN = 256


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


class PinnedArena:
    """First-fit allocator over one page-locked host buffer (allocated once).

    ``alloc`` returns an offset (bytes, 256-aligned) or None when no free
    range is large enough; ``free`` returns a range and merges it with its
    free neighbours."""

    def __init__(self, nbytes, pinned=True):
        self.size = int(nbytes) // _ALIGN * _ALIGN
        self.buf = torch.empty(self.size, dtype=torch.uint8, pin_memory=pinned and self.size > 0)
        self.free_list = [(0, self.size)] if self.size else []  # sorted (offset, length)
        self.used = {}

    def alloc(self, nbytes):
        n = max(_ALIGN, (int(nbytes) + _ALIGN - 1) // _ALIGN * _ALIGN)
        for i, (off, ln) in enumerate(self.free_list):
            if ln >= n:
                if ln == n:
                    self.free_list.pop(i)
                else:
                    self.free_list[i] = (off + n, ln - n)
                self.used[off] = n
                return off
        return None

    def free(self, off):
        n = self.used.pop(off)
        i = bisect.bisect_left(self.free_list, (off, 0))
        self.free_list.insert(i, (off, n))
        if i + 1 < len(self.free_list) and off + n == self.free_list[i + 1][0]:  # merge with the next range
            self.free_list[i] = (off, n + self.free_list[i + 1][1])
            self.free_list.pop(i + 1)
        if i > 0 and self.free_list[i - 1][0] + self.free_list[i - 1][1] == off:  # and with the previous one
            self.free_list[i - 1] = (self.free_list[i - 1][0], self.free_list[i - 1][1] + self.free_list[i][1])
            self.free_list.pop(i)

    def view(self, off, shape, dtype):
        """Host tensor over [off, off + nbytes) of the arena."""
        n = int(np.prod(shape)) * torch.tensor([], dtype=dtype).element_size()
        return self.buf[off : off + n].view(dtype).view(*shape)

    @property
    def in_use(self):
        return sum(self.used.values())


def _staged_bytes(n):
    return max(_ALIGN, (int(n) + _ALIGN - 1) // _ALIGN * _ALIGN)


class _Group:
    """Requests launched together: one stream, one completion event."""

    def __init__(self, stream, reqs, nbytes):
        self.stream = stream
        self.reqs = reqs
        self.nbytes = nbytes
        self.event = torch.cuda.Event()
        self.keep = []
        self.host = []      # per request: pinned host view of its result
        self.staged = []    # arena offsets held by this group
        self.spill = []     # one-off pinned tensors (the arena was full)


class Server:
    """Request loop over resident interpolants (see the module docstring).

    ``memory_budget`` (GiB) bounds the device memory of the requests in
    flight; ``staging`` (GiB) is the size of the pinned host arena: size it
    for the inputs and outputs of the requests in flight, since a request that
    finds it full pins a one-off host buffer, and pinning a new buffer of a
    few hundred MB holds up every host thread's CUDA calls for tens of ms
    (``stats()["staging_spills"]`` counts them)."""

    def __init__(self, interpolants: dict, memory_budget: float = 8.0, n_streams: int = 8, staging: float = 1.0,
                 n_fast_streams: int = 4, fast_work: float = 2e11, host_threads: int = 4):
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
        self.arena = PinnedArena(int(staging * 1024**3))
        self.streams = [torch.cuda.Stream(device=self.dev) for _ in range(n_streams)]
        self.free_streams = collections.deque(self.streams)
        # highest priority of the device (out-of-range values map to it)
        self.fast_streams = [torch.cuda.Stream(device=self.dev, priority=-100) for _ in range(n_fast_streams)]
        self.free_fast = collections.deque(self.fast_streams)
        self.fast_work = float(fast_work)
        self.fast_launches = 0
        self.waiting = collections.deque()
        self.inflight = []
        self.lock = threading.Lock()
        self.completed = []
        self.rejected = []
        self.failed = []
        self.batch_launches = 0
        self.launches = 0
        self.admitted = 0
        self.spilled = 0
        self.pending = 0  # launches and completions handed to the host threads, not yet finished
        self._building = {}  # stream -> group of a launch being prepared
        self.pool = ThreadPoolExecutor(max_workers=host_threads) if host_threads > 0 else None

    def close(self):
        """Stop the host threads (after ``drain``)."""
        if getattr(self, "pool", None) is not None:
            self.pool.shutdown(wait=True)
            self.pool = None

    def _run(self, fn, *args):
        """fn(*args) on a host thread of the pool, or here without one."""
        if getattr(self, "pool", None) is None:
            fn(*args)
            return
        with self.lock:
            self.pending += 1

        def task():
            try:
                fn(*args)
            finally:
                with self.lock:
                    self.pending -= 1

        self.pool.submit(task)

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
            return not self.waiting and not self.inflight and not getattr(self, "pending", 0)

    def step(self):
        """One scheduling step: complete finished launches, then admit and launch."""
        self._poll()
        self._admit()

    def drain(self, timeout=600.0):
        t0 = time.perf_counter()
        while not self.idle():
            self.step()
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("server did not drain")
            time.sleep(0.0002)

    # ------------------------------------------------------------------ sizes
    def request_bytes(self, req):
        """Device bytes of one request: input, output and the scratch the
        kernels of its path allocate (from the library's workspace queries and
        the tensors the paths create)."""
        ip = self.ips[req.name]
        P, d_in, d_out = req.points, ip.d_in, ip.d_out
        sp = self.spec[req.name]
        b = P * d_in * 8
        if req.op == "grad":
            bwd = sp._bwd
            ldo, ldk = bwd["ldo"], bwd["ldk"]
            step = min(P, max(128, int(sp.memory_limit * 1024**3 // (8 * ldk)) // 128 * 128))
            b += P * d_out * 4 + 3 * P * ldo * 4 + P * d_in * 8  # cotangent, its TF32 split, dL/dx
            b += step * (ldk + 31) // 32 * 32 * 4 + capi.size("smx_spectral_vjp_x_workspace", bwd["n_slots"],
                                                               bwd["vjp_seg"][1], step)
        elif req.precision == "fp64" and ip._fp64_orthogonal() is not None:
            b += P * d_out * 8  # the FP64 orthogonal evaluator takes no scratch
        elif req.precision == "fp64":
            per_point = capi.size("smx_eval_workspace", ip._plan.ref(), 1, 64)
            b += P * d_out * 8 + capi.size("smx_eval_workspace", ip._plan.ref(), min(P, max(1, ip._chunk(per_point))),
                                           64)
        else:
            b += P * d_out * 4
            if sp.tc is not None:
                step = sp._tc_step(P)
                b += 2 * step * (sp.tc["K"] + 31) // 32 * 32 * 4 + capi.size("smx_spectral_panel_workspace",
                                                                               sp.tc["n_slots"], step)
                if sp.tc_splits() > 1:
                    b += capi.size("smx_gemm_tf32x3_splitk_workspace", step, d_out, sp.tc["K"], sp.tc_splits())
            elif sp.blocked is not None:
                b += self.sms * 2 * 16 * 128 * 4 + 4 * self.sms
        return int(b)

    def work(self, req):
        """Estimated multiply-adds of a request: points x |Lambda| x d_out (the
        orthogonal form's terms), x3 for a gradient (panel, contraction and
        its transpose), or the combination sum's entries x d_out for an FP64
        evaluation that runs it."""
        ip = self.ips[req.name]
        per = float(ip._tree.size) * ip.d_out
        if req.op == "grad":
            per *= 3.0
        elif req.precision == "fp64" and ip._fp64_orthogonal() is None:
            per = float(ip._plan.c.n_entries) * ip.d_out
        return req.points * per

    def _kind(self, req):
        """Launch kind: (fast, 'blocked' / 'stream') for the persistent
        multi-plan launches, or (fast, 'plan', name, op, precision[, id]) for
        requests evaluated by one call per interpolant; ``fast`` selects the
        high-priority streams."""
        sp = self.spec[req.name]
        fast = self.work(req) <= self.fast_work
        if req.op == "eval" and req.precision == "fp32" and sp.tc is None:
            if sp.blocked is None:
                return (fast, "stream")
            if req.points <= 128 * self.sms:
                return (fast, "blocked")
            # a blocked request of a full round of tiles or more fills the GPU
            # alone and is evaluated exactly as alone (last-round split)
            return (fast, "plan", req.name, req.op, req.precision, req.id)
        return (fast, "plan", req.name, req.op, req.precision)

    # ------------------------------------------------------------------ admission
    def _admit(self):
        batches = {}
        with self.lock:
            # streams not yet promised in this step, per class (normal, fast)
            avail = {False: len(self.free_streams), True: len(self.free_fast)}
            kept = collections.deque()
            while self.waiting:
                req = self.waiting.popleft()
                nb = self.request_bytes(req)
                if nb > self.budget:
                    req.error = "request needs %d bytes, more than the server's budget" % nb
                    req.t_done = time.perf_counter()
                    req.done.set()
                    self.rejected.append(req)
                    continue
                if self.in_use + nb > self.budget:
                    kept.append(req)
                    break
                kind = self._kind(req)
                if kind not in batches:
                    if avail[kind[0]] < 1:
                        kept.append(req)  # no stream of its class: later requests may still go
                        if not avail[True] and not avail[False]:
                            break
                        continue
                    avail[kind[0]] -= 1  # one stream per launch
                batches.setdefault(kind, []).append((req, nb))
                self.in_use += nb
                self.admitted += 1
            kept.extend(self.waiting)
            self.waiting = kept
            streams = {kind: (self.free_fast if kind[0] else self.free_streams).popleft() for kind in batches}
        now = time.perf_counter()
        for kind, batch in batches.items():
            self._run(self._prepare, kind, batch, streams[kind], now)

    def _prepare(self, kind, batch, stream, now):
        try:
            self._launch_batch(kind, batch, stream, now)
        except Exception as e:  # the launch could not be prepared: fail its requests, give back what it took
            self._fail(kind, batch, stream, e)

    def _fail(self, kind, batch, stream, exc):
        msg = "%s: %s" % (type(exc).__name__, exc)
        for req, _ in batch:
            req.error = msg
            req.t_done = time.perf_counter()
            req.done.set()
        with self.lock:
            g = getattr(self, "_building", {}).pop(stream, None)
        if g is not None and g.staged:
            stream.synchronize()  # copies already queued from or into its staging ranges have finished
        with self.lock:
            if g is not None:
                for off in g.staged:
                    self.arena.free(off)
            self.failed.extend(r for r, _ in batch)
            self.in_use -= sum(nb for _, nb in batch)
            self._release_stream(stream, kind[0])

    # ------------------------------------------------------------------ staging
    def _stage(self, g, nbytes):
        """Pinned host range of nbytes: from the arena, else a one-off pinned tensor."""
        with self.lock:
            off = self.arena.alloc(nbytes)
            if off is not None:
                g.staged.append(off)
        if off is not None:
            return lambda shape, dtype: self.arena.view(off, shape, dtype)
        t = torch.empty(_staged_bytes(nbytes), dtype=torch.uint8, pin_memory=True)
        g.spill.append(t)
        with self.lock:
            self.spilled += 1
        return lambda shape, dtype: t[: int(np.prod(shape)) * torch.tensor([], dtype=dtype).element_size()].view(
            dtype).view(*shape)

    def _h2d_into(self, g, req, dst):
        """Copy the request's input into the device rows dst (stream-ordered)."""
        view = self._stage(g, req.x.nbytes)(req.x.shape, torch.float64)
        view.copy_(torch.from_numpy(req.x))  # host copy on torch's intra-op threads
        dst.copy_(view, non_blocking=True)

    def _d2h(self, g, y):
        h = self._stage(g, y.numel() * y.element_size())(tuple(y.shape), y.dtype)
        h.copy_(y, non_blocking=True)
        g.host.append(h)

    # ------------------------------------------------------------------ launches
    def _launch_batch(self, kind, batch, stream, now):
        g = _Group(stream, [r for r, _ in batch], sum(nb for _, nb in batch))
        g.fast = kind[0]
        with self.lock:
            self._building[stream] = g
        with torch.cuda.device(self.dev), torch.cuda.stream(stream):
            for req, _ in batch:
                req.t_admit = now
            if kind[1] in ("blocked", "stream"):
                self._launch_multiplan(kind[1], batch, g)
            else:
                self._launch_plan(kind[1:], batch, g)
            g.event.record(stream)
        with self.lock:
            self._building.pop(stream, None)
            self.launches += 1
            self.fast_launches += int(kind[0])
            self.batch_launches += int(kind[1] in ("blocked", "stream") or len(batch) > 1)
            self.inflight.append(g)

    def _release_stream(self, stream, fast):
        (self.free_fast if fast else self.free_streams).append(stream)

    def _launch_multiplan(self, kind, batch, g):
        plan_idx, plans = {}, []
        for req, _ in batch:
            if req.name not in plan_idx:
                plan_idx[req.name] = len(plans)
                sp = self.spec[req.name]
                plans.append(sp.blocked if kind == "blocked" else sp.c)
        struct = capi.SmxBlocked if kind == "blocked" else capi.SmxSpectral
        arr = (struct * len(plans))(*plans)
        items = (capi.SmxWork * len(batch))()
        outs = []
        for i, (req, _) in enumerate(batch):
            xd = torch.empty(req.x.shape, dtype=torch.float64, device=self.dev)
            self._h2d_into(g, req, xd)
            y = torch.empty(req.points, self.ips[req.name].d_out, dtype=torch.float32, device=self.dev)
            g.keep += [xd, y]
            outs.append(y)
            items[i].plan = plan_idx[req.name]
            items[i].x = xd.data_ptr()
            items[i].P = req.points
            items[i].ldx = req.x.shape[1]
            items[i].y = y.data_ptr()
        if kind == "blocked":
            nws = capi.size("smx_blocked_eval_batch_workspace", len(plans), len(batch))
        else:
            nws = capi.size("smx_spectral_eval_batch_workspace", len(plans), len(batch), max(p.d_out for p in plans))
        ws = torch.empty(nws, dtype=torch.uint8, device=self.dev)
        g.keep.append(ws)
        fn = "smx_blocked_eval_batch" if kind == "blocked" else "smx_spectral_eval_batch"
        call(fn, arr, len(plans), items, len(batch), ptr(ws), ws.numel(), capi.stream_ptr(g.stream))
        for y in outs:
            self._d2h(g, y)

    def _launch_plan(self, kind, batch, g):
        """Requests of one interpolant, operation and precision: one call over
        their concatenated points."""
        name, op, prec = kind[1], kind[2], kind[3]
        ip = self.ips[name]
        sizes = [req.points for req, _ in batch]
        offs = np.concatenate([[0], np.cumsum(sizes)])
        xd = torch.empty(int(offs[-1]), ip.d_in, dtype=torch.float64, device=self.dev)
        for (req, _), a, b in zip(batch, offs[:-1], offs[1:]):
            self._h2d_into(g, req, xd[a:b])
        g.keep.append(xd)
        if op == "eval":
            y = ip(xd, precision=prec)
        else:
            cot = torch.empty(int(offs[-1]), ip.d_out, dtype=torch.float32, device=self.dev)
            for (req, _), a, b in zip(batch, offs[:-1], offs[1:]):
                if req.cotangent is None:
                    cot[a:b] = 1.0
                else:
                    cot[a:b] = torch.as_tensor(np.asarray(req.cotangent, dtype=np.float32)).to(self.dev)
            y, _ = self.spec[name].vjp(xd, cot, need_x=True, need_coef=False, check=False)
            g.keep.append(cot)
        g.keep.append(y)
        for a, b in zip(offs[:-1], offs[1:]):
            self._d2h(g, y[a:b])

    # ------------------------------------------------------------------ completion
    def _poll(self):
        with self.lock:
            done = [g for g in self.inflight if g.event.query()]
            for g in done:
                self.inflight.remove(g)
        for g in done:
            self._run(self._complete, g)

    def _complete(self, g):
        """Hand a finished launch's results to its requests (a request is done
        when its result is in its own host array) and give back the launch's
        staging space, memory and stream."""
        failed = []
        for req, h in zip(g.reqs, g.host):
            try:
                out = torch.empty(tuple(h.shape), dtype=h.dtype)
                out.copy_(h)  # out of the staging arena, on torch's intra-op threads
                req.result = out.numpy()
            except Exception as e:  # the request fails; the launch's resources are still given back
                req.error = "%s: %s" % (type(e).__name__, e)
                failed.append(req)
            req.t_done = time.perf_counter()
            req.done.set()
        with self.lock:
            self.completed.extend(r for r in g.reqs if r not in failed)
            self.failed.extend(failed)
            for off in g.staged:
                self.arena.free(off)
            self.in_use -= g.nbytes
            self._release_stream(g.stream, g.fast)

    # ------------------------------------------------------------------ statistics
    def reset_stats(self):
        """Forget completed, rejected and failed requests and zero the launch
        counters (e.g. after a warm-up); requests in flight are unaffected."""
        with self.lock:
            self.completed, self.rejected, self.failed = [], [], []
            self.batch_launches = self.launches = self.fast_launches = self.admitted = self.spilled = 0

    def stats(self):
        lat = np.array([r.latency for r in self.completed]) if self.completed else np.zeros(1)
        evals = sum(r.points * self.ips[r.name].d_out for r in self.completed if r.op == "eval")
        return dict(
            completed=len(self.completed), rejected=len(self.rejected), failed=len(self.failed),
            launches=self.launches, batch_launches=self.batch_launches, fast_launches=self.fast_launches,
            staging_spills=self.spilled,
            p50_ms=float(np.percentile(lat, 50) * 1e3), p99_ms=float(np.percentile(lat, 99) * 1e3), evals=int(evals),
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
