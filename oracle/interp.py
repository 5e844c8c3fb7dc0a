"""Oracle restatement of the Smolyak interpolant (test infrastructure).

Follows ``src/smolyax/interpolation.py`` (block assembly in ``set_f``,
``__call__``, ``gradient``, ``integral``) and ``src/smolyax/barycentric.py``
(basis, tensor-product contraction, gradient).  The per-summand ``vmap`` of
the reference is replaced by batched numpy contractions over chunks of
summands and points; the arithmetic per summand is the reference's.
"""

from __future__ import annotations

import itertools as it
import string

import numpy as np

from . import indices as _indices
from . import nodes as _nodes


class OracleInterpolant:
    """Blocks of the reference's ``set_f`` plus evaluation (``interpolation.py:115-239``).

    ``rules`` is a list of per-dimension node rules (see ``oracle.nodes``);
    ``nested`` selects the f-evaluation cache layout of the reference (global
    keys for nested rules, per-multi-index dictionaries otherwise).
    """

    def __init__(self, *, rules, k, t, d_out, f, nested, f_evals=None):
        self.rules = list(rules)
        self.k = [float(v) for v in k]
        self.t = float(t)
        self.d_in = len(self.k)
        self.d_out = int(d_out)
        self.nested = bool(nested)
        self.n_f_evals_new = 0
        self.f_evals = self._assemble(f, {} if f_evals is None else f_evals)

    # -- set_f (interpolation.py:138-239) -------------------------------------------------
    def _assemble(self, f, f_evals):
        zero = np.array([_nodes.rule_nodes(r, 0)[0] for r in self.rules])
        n2nus, n2zetas = _indices.non_zero_indices_and_zetas(self.k, self.t)
        self.offset = 0
        self.blocks = {}
        for n, nus in n2nus.items():
            if n == 0:
                assert len(n2zetas[n]) == 1
                cache = f_evals if self.nested else f_evals.get((), {})
                if () not in cache:
                    cache[()] = f(zero.copy())
                    self.n_f_evals_new += 1
                if not self.nested:
                    f_evals[()] = cache
                self.offset = n2zetas[n][0] * np.asarray(cache[()], dtype=float)
                continue
            nn = len(nus)
            sdims = np.empty((nn, n), dtype=np.int64)
            sdegs = np.empty((nn, n), dtype=np.int64)
            for i, nu in enumerate(nus):
                srt = sorted(nu, key=lambda e: e[1], reverse=True)  # stable: ties keep ascending dim
                sdims[i] = [e[0] for e in srt]
                sdegs[i] = [e[1] for e in srt]
            tau = tuple(int(v) for v in sdegs.max(axis=0))
            m = max(tau) + 1
            xi = np.zeros((nn, n, m))
            wt = np.zeros((nn, n, m))
            for s in range(n):
                for i in range(nn):
                    dim, deg = int(sdims[i, s]), int(sdegs[i, s])
                    pts = _nodes.rule_nodes(self.rules[dim], deg)
                    xi[i, s, : deg + 1] = pts
                    wt[i, s, : deg + 1] = _nodes.barycentric_weights(pts)
            F = np.zeros((nn,) + tuple(v + 1 for v in tau) + (self.d_out,))
            for i, nu in enumerate(nus):
                cache = f_evals if self.nested else f_evals.get(nu, {})
                s_i = sdims[i]
                order = np.argsort(s_i)
                for mu in it.product(*[range(v + 1) for v in sdegs[i]]):
                    key = tuple((int(s_i[j]), int(mu[j])) for j in order if mu[j] > 0)
                    if key not in cache:
                        x = zero.copy()
                        x[s_i] = [xi[i, s, mu[s]] for s in range(n)]
                        cache[key] = f(x)
                        self.n_f_evals_new += 1
                    F[(i,) + tuple(mu)] = cache[key]
                if not self.nested:
                    f_evals[nu] = cache
            self.blocks[n] = dict(
                dims=sdims,
                degs=sdegs,
                nodes=xi,
                weights=wt,
                F=np.moveaxis(F, -1, 1).copy(),
                zetas=np.array(n2zetas[n], dtype=np.int64),
                tau=tau,
            )
        return f_evals

    # -- barycentric.py:34-66 ----------------------------------------------------------------
    @staticmethod
    def _basis(x, xi, w, deg):
        """Unnormalised basis with the one-hot exact-node rule; x (Z,P), xi/w (Z,m), deg (Z,)."""
        diffs = x[:, :, None] - xi[:, None, :]
        cols = np.arange(xi.shape[1])[None, :] <= deg[:, None]
        hit = np.any((diffs == 0) & cols[:, None, :], axis=2)
        one_hot = (diffs == 0).astype(float)
        with np.errstate(divide="ignore", invalid="ignore"):
            b = np.where(hit[:, :, None], one_hot, w[:, None, :] / diffs)
        return np.where(cols[:, None, :], b, 0.0)

    # -- barycentric.py:126-155 --------------------------------------------------------------
    @staticmethod
    def _basis_grad(x, xi, w, deg):
        diffs = (x[:, :, None] - xi[:, None, :]) ** 2
        cols = np.arange(xi.shape[1])[None, :] <= deg[:, None]
        sing = (diffs == 0) & cols[:, None, :]
        with np.errstate(divide="ignore", invalid="ignore"):
            v = np.where(sing, np.nan, -w[:, None, :] / diffs)
        return np.where(cols[:, None, :], v, 0.0)

    def _block_chunks(self, blk, zchunk):
        nn = blk["zetas"].shape[0]
        for z0 in range(0, nn, zchunk):
            yield slice(z0, min(nn, z0 + zchunk))

    # -- barycentric.py:69-123 and interpolation.py:264-304 ---------------------------------
    def __call__(self, x, *, pchunk=2048, zchunk=256, dtype=np.float64):
        """Evaluate at x.  ``dtype=np.longdouble`` evaluates the same formula in
        extended precision (nodes, weights and basis recomputed from the FP64
        nodes; nodal values are the FP64 data), which exposes the rounding
        error of FP64 evaluations of the combination sum."""
        x = np.asarray(x, dtype=float)
        if x.shape == (self.d_in,):
            x = x[None, :]
        assert x.shape[1] == self.d_in
        P = x.shape[0]
        out = np.broadcast_to(np.asarray(self.offset, dtype=float), (P, self.d_out)).astype(dtype)
        for n, blk in self.blocks.items():
            letters = string.ascii_lowercase
            fa = letters[:n]
            sub = "z,zo" + fa + "," + ",".join("zp" + c for c in fa) + "->po"
            for zs in self._block_chunks(blk, zchunk):
                dims, degs = blk["dims"][zs], blk["degs"][zs]
                for p0 in range(0, P, pchunk):
                    xp = x[p0 : p0 + pchunk].astype(dtype)
                    bs = []
                    for s in range(n):
                        m = blk["tau"][s] + 1
                        xi = blk["nodes"][zs, s, :m].astype(dtype)
                        w = blk["weights"][zs, s, :m].astype(dtype)
                        if dtype is not np.float64:
                            w = np.zeros_like(xi)
                            for z in range(xi.shape[0]):
                                g = int(degs[z, s])
                                w[z, : g + 1] = _nodes.barycentric_weights(xi[z, : g + 1], dtype=dtype)
                        b = self._basis(xp[:, dims[:, s]].T, xi, w, degs[:, s])
                        bs.append(b / b.sum(axis=2, keepdims=True))
                    F = blk["F"][zs].astype(dtype)
                    out[p0 : p0 + pchunk] += np.einsum(sub, blk["zetas"][zs].astype(dtype), F, *bs, optimize=True)
        return out

    # -- barycentric.py:158-229 and interpolation.py:306-345 --------------------------------
    def gradient(self, x, *, pchunk=512, zchunk=128, dtype=np.float64):
        x = np.asarray(x, dtype=float)
        if x.shape == (self.d_in,):
            x = x[None, :]
        P = x.shape[0]
        J = np.zeros((P, self.d_out, self.d_in), dtype=dtype)
        for n, blk in self.blocks.items():
            fa = string.ascii_lowercase[:n]
            for zs in self._block_chunks(blk, zchunk):
                dims, degs = blk["dims"][zs], blk["degs"][zs]
                zeta = blk["zetas"][zs].astype(dtype)
                for p0 in range(0, P, pchunk):
                    xp = x[p0 : p0 + pchunk].astype(dtype)
                    bn, Bd = [], []
                    for s in range(n):
                        m = blk["tau"][s] + 1
                        xs = xp[:, dims[:, s]].T
                        xi, w = blk["nodes"][zs, s, :m].astype(dtype), blk["weights"][zs, s, :m].astype(dtype)
                        if dtype is not np.float64:
                            w = np.zeros_like(xi)
                            for z in range(xi.shape[0]):
                                g = int(degs[z, s])
                                w[z, : g + 1] = _nodes.barycentric_weights(xi[z, : g + 1], dtype=dtype)
                        b = self._basis(xs, xi, w, degs[:, s])
                        bnorm = b.sum(axis=2, keepdims=True)
                        db = self._basis_grad(xs, xi, w, degs[:, s])
                        dbnorm = db.sum(axis=2, keepdims=True)
                        b = b / bnorm
                        bn.append(b)
                        Bd.append(db / bnorm - b * dbnorm / bnorm)
                    for s in range(n):
                        ops = [Bd[j] if j == s else bn[j] for j in range(n)]
                        sub = "z,zo" + fa + "," + ",".join("zp" + c for c in fa) + "->zpo"
                        g = np.einsum(sub, zeta, blk["F"][zs].astype(dtype), *ops, optimize=True)  # (Z, P, d_out)
                        for zi in range(g.shape[0]):
                            J[p0 : p0 + pchunk, :, dims[zi, s]] += g[zi]
        return J

    # -- interpolation.py:347-390 -------------------------------------------------------------
    def integral(self, dtype=np.float64):
        Q = np.broadcast_to(np.asarray(self.offset, dtype=float), (self.d_out,)).astype(dtype)
        for n, blk in self.blocks.items():
            nn = blk["zetas"].shape[0]
            qs = []
            for s in range(n):
                q = np.zeros((nn, blk["tau"][s] + 1), dtype=dtype)
                for i in range(nn):
                    dim, deg = int(blk["dims"][i, s]), int(blk["degs"][i, s])
                    q[i, : deg + 1] = _nodes.rule_quadrature_weights(self.rules[dim], deg)
                qs.append(q)
            fa = string.ascii_lowercase[:n]
            sub = "z," + ",".join("z" + c for c in fa) + ",zo" + fa + "->o"
            Q += np.einsum(sub, blk["zetas"].astype(dtype), *qs, blk["F"].astype(dtype), optimize=True)
        return Q

    # -- flattened view used by tests ------------------------------------------------------------
    def summands(self):
        """List of (sparse nu in ascending dim order, zeta) over all n >= 0."""
        n2nus, n2zetas = _indices.non_zero_indices_and_zetas(self.k, self.t)
        out = []
        for n in n2nus:
            out.extend(zip(n2nus[n], n2zetas[n]))
        return out


def rules_from_spec(kind, d, domains=None, mean=None, scaling=None):
    """Per-dimension rule tuples for ``OracleInterpolant``."""
    if kind == "leja":
        if domains is None:
            return [("leja", None)] * d
        return [("leja", (float(a), float(b))) for a, b in domains]
    mean = np.zeros(d) if mean is None else np.asarray(mean, dtype=float)
    scaling = np.ones(d) if scaling is None else np.asarray(scaling, dtype=float)
    return [("gh", (float(m), float(s))) for m, s in zip(mean, scaling)]

