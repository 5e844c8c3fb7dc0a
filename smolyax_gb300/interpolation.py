r"""Barycentric Smolyak interpolant on the GPU (mirrors ``src/smolyax/interpolation.py``).

$I^{\Lambda_{k,t}}[f] = \sum_{\nu\in\Lambda} \zeta_{\Lambda,\nu} I^\nu[f]$.  Set-up
(``set_f``) builds the index set, the Smolyak coefficients and the summand
layout on the device, calls the user function at every interpolation node on
the host (the reference's f-evaluation cache format is kept), and gathers the
nodal values into an unpadded device array.  Evaluation, gradient and
integral run as hand-written sm_103a kernels through the C ABI.
"""
from __future__ import annotations

import math
from typing import Callable, Sequence, Union

import numpy as np
import torch

from . import _capi as capi
from . import indices
from . import nodes as _nodes
from ._capi import call, ptr

ArrayLike = Union[np.ndarray, torch.Tensor]

# host inputs of at least this many rows are copied and evaluated in overlapped chunks (FP32)
_OVERLAP_MIN_ROWS = 16384
_PRECISIONS = ("fp64", "fp64_barycentric", "fp32")


def _stream():
    return capi.stream_ptr(torch.cuda.current_stream())


class Plan:
    """Device arrays of one interpolant plus the C struct that points at them."""

    def __init__(self):
        self.keep = {}
        self.c = capi.SmxPlan()

    def set(self, name, tensor):
        self.keep[name] = tensor
        if hasattr(self.c, name):
            setattr(self.c, name, None if tensor is None else tensor.data_ptr())

    def ref(self):
        import ctypes

        return ctypes.byref(self.c)


class SmolyakBarycentricInterpolator:
    r"""Smolyak operator for $f:\mathbb R^{d_{in}}\to\mathbb R^{d_{out}}$ (``interpolation.py:15-113``).

    Same keyword-only constructor as the reference.  Results are torch tensors
    on the CUDA device; inputs may be numpy arrays or torch tensors.
    """

    @property
    def d_in(self) -> int:
        return self._d_in

    @property
    def d_out(self) -> int:
        return self._d_out

    @property
    def n_f_evals(self) -> int:
        return self._n_f_evals

    @property
    def n_f_evals_new(self) -> int:
        return self._n_f_evals_new

    def __init__(self, *, d_out: int, node_gen: _nodes.Generator, k: Sequence[float], t: float,
                 f: Callable = None, n_inputs: int = None, memory_limit: float = 4.0,
                 precision: str = "fp64") -> None:
        """Keyword arguments as in the reference (``interpolation.py:51-113``), plus
        ``precision``: "fp64" (default) evaluates in FP64 -- plans over Leja /
        Gauss-Hermite rules in the orthogonal-polynomial form (coefficients from
        compensated FP64 sums; ~1e-14 relative to the exact value, ~10x faster),
        other rules as the reference's combination sum;
        "fp64_barycentric" always evaluates the combination sum (the reference's
        algorithm, interpolation.py:264-304); "fp32" evaluates the orthogonal form
        in FP32 and returns FP32 values."""
        if precision not in _PRECISIONS:
            raise ValueError("precision must be one of " + ", ".join(repr(v) for v in _PRECISIONS))
        self._precision = precision
        self._spectral = None
        self._fp64_form_ok = None
        self._side_streams = {}  # device -> the two streams of chunked host-input evaluation
        self._d_in = len(k)
        self._d_out = int(d_out)
        self._node_gen = node_gen
        self._is_nested = node_gen.is_nested
        self._k = np.asarray(k, dtype=np.float64)
        self._t = float(t)
        self._memory_limit = float(memory_limit)
        self._n_inputs = n_inputs
        self._plan = None
        self._n_f_evals = indices.nodeset_cardinality(self._k, self._t, nested=self._is_nested)
        self._n_f_evals_new = 0
        if f is not None:
            self.set_f(f=f)

    # ------------------------------------------------------------------ set-up
    def set_f(self, *, f: Callable, f_evals: dict = None) -> dict:
        """Evaluate (or reuse) f at the interpolation nodes and build the device plan
        (``interpolation.py:115-239``).  Returns the updated f-evaluation dictionary.

        By default f is called on the host as in the reference: with one point
        of shape (d_in,) at a time, or, if f has a true attribute
        ``vectorized``, once with the stacked [n, d_in] array of the missing
        nodes.  If f has a true attribute ``on_device``, it is called with CUDA
        tensors [n, d_in] (FP64) of node points, in chunks, and must return
        [n, d_out] tensors on the device; the nodal values then stay on the
        device and are not added to ``f_evals`` (the dictionary is returned
        unchanged and its entries are not reused)."""
        if f_evals is None:
            f_evals = {}
        dev = indices.device()
        st = _stream()
        gen = self._node_gen
        d, d_out = self._d_in, self._d_out
        zero = np.array([g(0)[0] for g in gen])

        tree = indices.LambdaTree(self._k, self._t, capi.SMX_MODE_NONZERO)
        zeta = tree.zeta()
        rank = tree.rank()
        level = tree.level_of()
        # summands: zeta != 0 and n >= 1, in the reference's emission order
        sel = torch.nonzero((zeta != 0) & (level >= 1)).flatten()
        ent = sel[torch.argsort(rank[sel])].contiguous()
        n_sum = int(ent.shape[0])
        zeta0 = int(zeta[0].item())

        # offset: zeta_0 * f(zero point)   (interpolation.py:151-166)
        if self._is_nested:
            cache0 = f_evals
        else:
            cache0 = f_evals.get((), {})
        on_device = bool(getattr(f, "on_device", False))
        zero_val = None
        if zeta0 != 0:
            if on_device:
                zero_val = torch.as_tensor(f(torch.as_tensor(zero[None, :], device=dev)), device=dev).to(
                    torch.float64).reshape(-1)
                cache0 = {(): zero_val.cpu().numpy()}
                self._n_f_evals_new += 1
            elif () not in cache0:
                cache0[()] = f(zero.copy())
                self._n_f_evals_new += 1
            if not self._is_nested and not on_device:
                f_evals[()] = cache0
            offset = zeta0 * self._as_out(cache0[()])
        else:
            offset = np.zeros(d_out)

        # pairs: every (dim, deg) with 1 <= deg <= maxdeg(dim)
        maxdeg = torch.zeros(d, dtype=torch.int32, device=dev)
        call("smx_max_degree", tree.size, ptr(tree.dim), ptr(tree.deg), ptr(maxdeg), st)
        maxdeg_h = maxdeg.cpu().numpy().astype(np.int64)
        pair_base_h = np.concatenate([[0], np.cumsum(maxdeg_h)[:-1]]).astype(np.int32)
        n_pairs = int(maxdeg_h.sum())
        pair_dim_h = np.repeat(np.arange(d, dtype=np.int32), maxdeg_h)
        pair_deg_h = (np.arange(n_pairs) - np.repeat(pair_base_h, maxdeg_h) + 1).astype(np.int32)
        pair_voff_h = np.concatenate([[0], np.cumsum(pair_deg_h + 1)[:-1]]).astype(np.int32)
        n_values = int((pair_deg_h + 1).sum())
        node_h = np.empty(n_values)
        for u in range(n_pairs):
            g = int(pair_deg_h[u])
            node_h[pair_voff_h[u] : pair_voff_h[u] + g + 1] = np.asarray(gen[int(pair_dim_h[u])](g), dtype=float)

        P = Plan()
        T = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
        P.set("pair_dim", T(pair_dim_h, torch.int32))
        P.set("pair_deg", T(pair_deg_h, torch.int32))
        P.set("pair_voff", T(pair_voff_h, torch.int32))
        P.set("node", T(node_h, torch.float64))
        bw = torch.empty(n_values, dtype=torch.float64, device=dev)
        call("smx_bary_weights", n_pairs, ptr(P.keep["pair_deg"]), ptr(P.keep["pair_voff"]), ptr(P.keep["node"]),
             ptr(bw), st)
        P.set("bweight", bw)

        # summand layout
        lvl_sum = level[ent]
        sum_poff = torch.zeros(n_sum + 1, dtype=torch.int32, device=dev)
        if n_sum:
            sum_poff[1:] = torch.cumsum(lvl_sum, 0).to(torch.int32)
        n_pair_tot = int(sum_poff[-1].item()) if n_sum else 0
        sum_pairs = torch.empty(max(n_pair_tot, 1), dtype=torch.int32, device=dev)
        n_ent = torch.empty(max(n_sum, 1), dtype=torch.int64, device=dev)
        pair_base = T(pair_base_h, torch.int32)
        call("smx_plan_summands", n_sum, ptr(ent), ptr(tree.parent), ptr(tree.dim), ptr(tree.deg), ptr(pair_base),
             ptr(sum_poff), ptr(sum_pairs), ptr(n_ent), st)
        sum_eoff = torch.empty(n_sum + 1, dtype=torch.int64, device=dev)
        ws = torch.empty(capi.size("smx_scan_workspace", n_sum), dtype=torch.uint8, device=dev)
        call("smx_scan_i64", ptr(n_ent), ptr(sum_eoff), n_sum, ptr(ws), ws.numel(), st)
        R = int(sum_eoff[-1].item())
        P.set("sum_poff", sum_poff)
        P.set("sum_pairs", sum_pairs)
        P.set("sum_eoff", sum_eoff)

        # nodal values: calls of f with the reference's cache keys, device gather
        if on_device:
            fu_d, umap = self._evaluate_nodes_on_device(f, zero, sum_poff.cpu().numpy(), sum_pairs.cpu().numpy(),
                                                        pair_dim_h, pair_deg_h, pair_voff_h, node_h, R, dev,
                                                        zero_val if self._is_nested else None)
        else:
            fu, umap = self._evaluate_nodes(f, f_evals, zero, sum_poff.cpu().numpy(), sum_pairs.cpu().numpy(),
                                            pair_dim_h, pair_deg_h, pair_voff_h, node_h, R)
        P.set("F64", torch.empty(max(R * d_out, 1), dtype=torch.float64, device=dev))
        P.set("F32", torch.empty(max(R * d_out, 1), dtype=torch.float32, device=dev))
        c = P.c
        c.d_in, c.d_out = d, d_out
        c.n_pairs, c.n_values, c.n_summands = n_pairs, n_values, n_sum
        c.max_n = int(lvl_sum.max().item()) if n_sum else 0
        c.n_entries = R
        P.keep["sum_zeta"] = zeta[ent].contiguous()
        P.keep["zeta0"] = zeta0
        P.keep["umap"] = T(umap, torch.int64)
        P.keep["offset0"] = T(offset, torch.float64)  # zeta_0 f(zero) as the reference computes it
        self._plan = P
        self._assemble_rows(fu_d if on_device else T(fu, torch.float64))
        P.keep["ent"] = ent
        self._spectral = None
        self._fp64_form_ok = None
        self._tree = tree
        self._maxdeg = maxdeg_h
        if self._n_inputs is not None:
            _ = self(torch.rand(self._n_inputs, d, dtype=torch.float64, device=dev))
        return f_evals

    def _assemble_rows(self, fu_d):
        """Device rows of the plan from the unique nodal values fu [U, d_out].

        Centering: every tensor-product interpolant reproduces constants, so
        sum_s zeta_s I^nu_s[f] = c * sum_s zeta_s + sum_s zeta_s I^nu_s[f - c].
        With c = f(zero point) (row 0 of every summand) the summands that
        cancel in the combination sum shrink by about an order of magnitude."""
        P = self._plan
        c = P.c
        R, d_out = c.n_entries, c.d_out
        fu_d = fu_d.reshape(-1, d_out).contiguous()
        P.keep["fu"] = fu_d
        if R:
            umap = P.keep["umap"]
            center = fu_d[umap[0]].clone()
            zsum = float(P.keep["sum_zeta"].sum().item())
            offset = P.keep["offset0"] + center * zsum
            P.keep["center"] = center
            P.set("offset", offset.contiguous())
            call("smx_assemble_F", P.ref(), ptr(P.keep["sum_zeta"]), ptr(fu_d), ptr(umap), ptr(center),
                 ptr(P.keep["F64"]), ptr(P.keep["F32"]), _stream())
        else:
            P.keep["center"] = torch.zeros(d_out, dtype=torch.float64, device=fu_d.device)
            P.set("offset", P.keep["offset0"].clone())
        self._spectral = None

    @property
    def nodal_values(self) -> torch.Tensor:
        """Unique function values at the interpolation nodes, [U, d_out] FP64 on the
        device (the rows the interpolant is built from; see ``set_nodal_values``)."""
        assert self._plan is not None, "The operator has not yet been set up for a target function via `set_f`."
        return self._plan.keep["fu"]

    def set_nodal_values(self, fu) -> None:
        """Rebuild the interpolant from new values at the same nodes (no calls of f)."""
        dev = indices.device()
        fu = torch.as_tensor(fu, dtype=torch.float64, device=dev)
        assert tuple(fu.shape) == tuple(self.nodal_values.shape), "nodal values must keep their shape"
        if self._plan.keep["zeta0"] != 0 and self._plan.c.n_entries:
            # the constant term follows the zero point's value in fu
            u0 = int(self._plan.keep["umap"][0].item())
            self._plan.keep["offset0"] = self._plan.keep["zeta0"] * fu[u0].clone()
        self._assemble_rows(fu)

    def _as_out(self, v):
        return np.broadcast_to(np.asarray(v, dtype=float), (self._d_out,)).astype(float)

    def _evaluate_nodes(self, f, f_evals, zero, sum_poff, sum_pairs, pdim, pdeg, pvoff, node, R):
        """Unique function values and the row -> value map (``interpolation.py:201-228``).

        Keys follow the reference's cache: nested rules key by the sparse node
        multi-index ((dim, mu), ...), non-nested rules by that key inside a
        dictionary per multi-index nu.  Missing values are computed by calling f
        once per node (the reference's convention) or, if f has a true attribute
        ``vectorized``, once on the stacked [n, d_in] array of missing nodes."""
        nested = self._is_nested
        vectorized = bool(getattr(f, "vectorized", False))
        keys = {}
        vals = []
        umap = np.empty(R, dtype=np.int64)
        pending = []  # (cache, key, point) of values still to compute
        pending_keys = set()
        rows = []  # (cache, key) per row
        r = 0
        n_sum = len(sum_poff) - 1
        for s in range(n_sum):
            prs = sum_pairs[sum_poff[s] : sum_poff[s + 1]]
            dims = [int(pdim[u]) for u in prs]
            degs = [int(pdeg[u]) for u in prs]
            offs = [int(pvoff[u]) for u in prs]
            if nested:
                cache = f_evals
                ukey = None
            else:
                nu = tuple(zip(dims, degs))
                cache = f_evals.get(nu, {})
                f_evals[nu] = cache
                ukey = nu
            n = len(dims)
            mu = [0] * n
            K = int(np.prod([g + 1 for g in degs]))
            for _ in range(K):
                key = tuple((dims[i], mu[i]) for i in range(n) if mu[i] > 0)
                if key not in cache and (ukey, key) not in pending_keys:
                    x = zero.copy()
                    for i in range(n):
                        x[dims[i]] = node[offs[i] + mu[i]]
                    pending.append((cache, key, x))
                    pending_keys.add((ukey, key))
                rows.append((cache, ukey, key))
                r += 1
                for i in range(n - 1, -1, -1):
                    mu[i] += 1
                    if mu[i] <= degs[i]:
                        break
                    mu[i] = 0
        if pending:
            if vectorized:
                out = np.asarray(f(np.stack([p[2] for p in pending])), dtype=float).reshape(len(pending), -1)
                for (cache, key, _), v in zip(pending, out):
                    cache[key] = v
            else:
                for cache, key, x in pending:
                    cache[key] = f(x)
            self._n_f_evals_new += len(pending)
        for r, (cache, ukey, key) in enumerate(rows):
            gk = (ukey, key)
            idx = keys.get(gk)
            if idx is None:
                idx = len(vals)
                keys[gk] = idx
                vals.append(self._as_out(cache[key]))
            umap[r] = idx
        fu = np.array(vals, dtype=float).reshape(-1, self._d_out) if vals else np.zeros((1, self._d_out))
        return fu, umap

    def _evaluate_nodes_on_device(self, f, zero, sum_poff, sum_pairs, pdim, pdeg, pvoff, node, R, dev,
                                  zero_val=None, chunk=1 << 16):
        """Unique nodal values computed by a device function f, and the row ->
        value map.  The unique nodes are found with the same keys as
        ``_evaluate_nodes`` (one per sparse node multi-index for nested rules,
        per multi-index nu and node otherwise), each recorded sparsely as the
        (dimension, node value) pairs of its summand; dense [chunk, d_in] point
        arrays are then assembled on the device (the zero point, with those
        coordinates scattered in) and passed to f.  ``zero_val``: f at the zero
        point, already evaluated for the offset (nested rules, where the node
        with key () is that point): reused and not counted again, as the host
        path finds it in its cache."""
        nested = self._is_nested
        index = {}
        umap = np.empty(R, dtype=np.int64)
        pt_len, pt_dims, pt_vals = [], [], []
        r = 0
        for s in range(len(sum_poff) - 1):
            prs = sum_pairs[sum_poff[s] : sum_poff[s + 1]]
            dims = [int(pdim[u]) for u in prs]
            degs = [int(pdeg[u]) for u in prs]
            offs = [int(pvoff[u]) for u in prs]
            nu = None if nested else tuple(zip(dims, degs))
            n = len(dims)
            mu = [0] * n
            for _ in range(int(np.prod([g + 1 for g in degs]))):
                gk = (nu, tuple((dims[i], mu[i]) for i in range(n) if mu[i] > 0))
                idx = index.get(gk)
                if idx is None:
                    idx = index[gk] = len(pt_len)
                    pt_len.append(n)
                    pt_dims.extend(dims)
                    pt_vals.extend(node[offs[i] + mu[i]] for i in range(n))
                umap[r] = idx
                r += 1
                for i in range(n - 1, -1, -1):
                    mu[i] += 1
                    if mu[i] <= degs[i]:
                        break
                    mu[i] = 0
        U = len(pt_len)
        reuse = index.get((None, ())) if zero_val is not None else None
        self._n_f_evals_new += U - (1 if reuse is not None else 0)
        fu = torch.empty(max(U, 1), self._d_out, dtype=torch.float64, device=dev)
        if U == 0:
            fu.zero_()
            return fu, umap
        lens = np.asarray(pt_len, dtype=np.int64)
        starts = np.concatenate([[0], np.cumsum(lens)])
        pt_dims = torch.as_tensor(np.asarray(pt_dims, dtype=np.int64), device=dev)
        pt_vals = torch.as_tensor(np.asarray(pt_vals, dtype=np.float64), device=dev)
        zero_d = torch.as_tensor(zero, dtype=torch.float64, device=dev)
        for u0 in range(0, U, chunk):
            u1 = min(U, u0 + chunk)
            a, b = int(starts[u0]), int(starts[u1])
            X = zero_d.repeat(u1 - u0, 1)
            rows = torch.as_tensor(np.repeat(np.arange(u1 - u0), lens[u0:u1]), device=dev)
            X[rows, pt_dims[a:b]] = pt_vals[a:b]
            out = torch.as_tensor(f(X), device=dev).to(torch.float64).reshape(u1 - u0, -1)
            if out.shape[1] != self._d_out:
                raise ValueError("f returned %d outputs per point, expected d_out = %d" % (out.shape[1], self._d_out))
            fu[u0:u1] = out
        if reuse is not None:
            fu[reuse] = zero_val
        return fu, umap

    # ------------------------------------------------------------------ evaluation
    def _validate_input(self, x: ArrayLike) -> torch.Tensor:
        """``interpolation.py:253-262``: set-up check, host->device, 1-D promotion."""
        assert self._plan is not None, "The operator has not yet been set up for a target function via `set_f`."
        dev = indices.device()
        if isinstance(x, torch.Tensor):
            x = x.to(device=dev, dtype=torch.float64)
        else:
            x = torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev)
        if tuple(x.shape) == (self._d_in,):
            x = x[None, :]
        assert x.shape[1] == self._d_in, f"{x.shape[1]} != {self._d_in}"
        self._n_inputs = int(x.shape[0])
        return x.contiguous()

    def _host_rows(self, x):
        """Rows of a 2-D host input of width d_in (0 for device inputs and other shapes)."""
        if isinstance(x, torch.Tensor):
            return int(x.shape[0]) if x.device.type == "cpu" and x.dim() == 2 and x.shape[1] == self._d_in else 0
        if isinstance(x, np.ndarray) and x.ndim == 2 and x.shape[1] == self._d_in:
            return int(x.shape[0])
        return 0

    def _call_fp32_host(self, x):
        """FP32 evaluation of a large host input: the rows are copied in chunks on
        two side streams, each chunk evaluated as soon as it has arrived, so the
        host->device transfer (the bound of this call) overlaps the evaluation."""
        assert self._plan is not None, "The operator has not yet been set up for a target function via `set_f`."
        xh = x if isinstance(x, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64))
        xh = xh.to(torch.float64).contiguous()
        Pn = int(xh.shape[0])
        self._n_inputs = Pn
        sp = self.spectral_plan()
        dev = indices.device()
        xd = torch.empty(Pn, self._d_in, dtype=torch.float64, device=dev)
        y = torch.empty(Pn, self._d_out, dtype=torch.float32, device=dev)
        cur = torch.cuda.current_stream(dev)
        # two side streams, created once per device
        streams = self._side_streams.get(dev)
        if streams is None:
            streams = self._side_streams[dev] = [torch.cuda.Stream(device=dev) for _ in range(2)]
        n_chunks = max(2, min(8, Pn // (_OVERLAP_MIN_ROWS // 2)))
        step = -(-Pn // n_chunks)
        for i, p0 in enumerate(range(0, Pn, step)):
            p1 = min(Pn, p0 + step)
            s = streams[i % 2]
            s.wait_stream(cur)
            with torch.cuda.stream(s):
                xd[p0:p1].copy_(xh[p0:p1], non_blocking=True)
                sp.evaluate(xd[p0:p1], y[p0:p1])
        for s in streams:
            cur.wait_stream(s)
            xd.record_stream(s)
            y.record_stream(s)
        return y

    def _chunk(self, bytes_per_point):
        lim = max(1, int(self._memory_limit * 1024**3 // max(1, bytes_per_point)))
        return lim

    def spectral_plan(self):
        """The FP32 orthogonal-polynomial form of this interpolant (built on first use)."""
        assert self._plan is not None, "The operator has not yet been set up for a target function via `set_f`."
        if self._spectral is None:
            from .spectral import SpectralPlan

            self._spectral = SpectralPlan(self)
        return self._spectral

    def __call__(self, x: ArrayLike, precision: str = None) -> torch.Tensor:
        """Evaluate the interpolant at points x, shape (n_points, d_in) or (d_in,) -> (n_points, d_out).

        ``precision`` overrides the constructor's choice for this call; "bf16x3"
        (plans with 16 or more outputs) runs the contraction with split-BF16
        operands (error bound 1e-4 relative, FP32 results)."""
        if precision is not None and precision not in _PRECISIONS + ("bf16x3",):
            raise ValueError("precision must be one of " + ", ".join(repr(v) for v in _PRECISIONS + ("bf16x3",)))
        if (precision or self._precision) == "fp32" and self._host_rows(x) >= _OVERLAP_MIN_ROWS:
            return self._call_fp32_host(x)
        x = self._validate_input(x)
        Pn = int(x.shape[0])
        if precision == "bf16x3":
            sp = self.spectral_plan()
            if sp.tc is None:
                raise ValueError("precision='bf16x3' needs the tensor-core form (16 or more outputs)")
            y16 = torch.empty(Pn, self._d_out, dtype=torch.float32, device=x.device)
            return sp.evaluate(x, y16, mode="bf16x3") if Pn else y16
        if (precision or self._precision) == "fp32":
            sp = self.spectral_plan()
            y32 = torch.empty(Pn, self._d_out, dtype=torch.float32, device=x.device)
            return sp.evaluate(x, y32) if Pn else y32
        y = torch.empty(Pn, self._d_out, dtype=torch.float64, device=x.device)
        if Pn == 0:
            return y
        if (precision or self._precision) == "fp64":
            sp = self._fp64_orthogonal()
            if sp is not None:
                return sp.evaluate64(x, y)
        st = _stream()
        pl = self._plan
        per_point = capi.size("smx_eval_workspace", pl.ref(), 1, 64)
        step = self._chunk(per_point)
        for p0 in range(0, Pn, step):
            p1 = min(Pn, p0 + step)
            ws = torch.empty(capi.size("smx_eval_workspace", pl.ref(), p1 - p0, 64), dtype=torch.uint8, device=x.device)
            call("smx_eval", pl.ref(), 64, ptr(x[p0:p1]), p1 - p0, self._d_in, ptr(y[p0:p1]), ptr(ws), ws.numel(), st)
        return y

    def _fp64_orthogonal(self):
        """The orthogonal form that FP64 evaluation uses, or None: Leja or
        Gauss-Hermite rules in every dimension (their polynomial families are the
        form's), degrees within the recurrence tables, and a per-point row of
        the FP64 evaluator within shared memory."""
        if self._fp64_form_ok is None:
            from .spectral import MAX_DEGREE

            self._fp64_form_ok = (int(np.max(self._maxdeg, initial=0)) < MAX_DEGREE
                                  and all(isinstance(g, (_nodes.Leja1D, _nodes.GaussHermite1D))
                                          for g in self._node_gen)
                                  and self.spectral_plan().fp64_form() is not None)
        return self.spectral_plan() if self._fp64_form_ok else None

    def gradient(self, x: ArrayLike) -> torch.Tensor:
        """Jacobian of the interpolant at x: (n_points, d_out, d_in) (``interpolation.py:306-345``)."""
        x = self._validate_input(x)
        Pn = int(x.shape[0])
        J = torch.empty(Pn, self._d_out, self._d_in, dtype=torch.float64, device=x.device)
        if Pn == 0:
            return J
        st = _stream()
        pl = self._plan
        per_point = capi.size("smx_jacobian_workspace", pl.ref(), 1)
        step = self._chunk(per_point)
        for p0 in range(0, Pn, step):
            p1 = min(Pn, p0 + step)
            ws = torch.empty(capi.size("smx_jacobian_workspace", pl.ref(), p1 - p0), dtype=torch.uint8,
                             device=x.device)
            call("smx_jacobian", pl.ref(), ptr(x[p0:p1]), p1 - p0, self._d_in, ptr(J[p0:p1]), ptr(ws), ws.numel(), st)
        return J

    def integral(self) -> torch.Tensor:
        """Integral of the interpolant, shape (d_out,) (``interpolation.py:347-390``)."""
        assert self._plan is not None, "The operator has not yet been set up for a target function via `set_f`."
        pl = self._plan
        dev = indices.device()
        c = pl.c
        if "qnode" not in pl.keep:
            pdim = pl.keep["pair_dim"].cpu().numpy()
            pdeg = pl.keep["pair_deg"].cpu().numpy()
            pvoff = pl.keep["pair_voff"].cpu().numpy()
            q = np.zeros(max(c.n_values, 1))
            for u in range(c.n_pairs):
                g = int(pdeg[u])
                q[pvoff[u] : pvoff[u] + g + 1] = self._node_gen[int(pdim[u])].get_quadrature_weights(g)
            pl.keep["qnode"] = torch.as_tensor(q, device=dev)
        Q = torch.empty(self._d_out, dtype=torch.float64, device=dev)
        ws = torch.empty(capi.size("smx_integral_workspace", pl.ref()), dtype=torch.uint8, device=dev)
        call("smx_integral", pl.ref(), ptr(pl.keep["qnode"]), ptr(Q), ptr(ws), ws.numel(), _stream())
        return Q
