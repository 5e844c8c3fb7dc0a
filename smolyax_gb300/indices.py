r"""Anisotropic multi-index sets on the GPU (mirrors ``src/smolyax/indices.py``).

$\Lambda_{k,t} = \{\nu \in \mathbb N_0^d : \sum_j k_j \nu_j < t\}$ is built level by
level on the device: level n holds the multi-indices with n non-zero entries,
each entry carrying the remaining budget after its last inclusion.  The
floating-point decisions are the reference's, operation for operation, so the
sets, their order and the Smolyak coefficients are bit-identical to the
reference's numba/Python results.  The public functions keep the reference's
names, arguments and return types.
"""
from __future__ import annotations

from collections import defaultdict
from typing import Sequence

import numpy as np
import torch

from . import _capi as capi
from ._capi import call, ptr


def device():
    """The CUDA device used by the library (raises without one: there is no CPU path)."""
    if not torch.cuda.is_available():
        raise RuntimeError("smolyax_gb300 needs a CUDA GPU (GB300, sm_103a); no CPU fallback exists")
    return torch.device("cuda", torch.cuda.current_device())


def _stream():
    return capi.stream_ptr(torch.cuda.current_stream())


class LambdaTree:
    """Device-resident enumeration of Lambda_{k,t} in one of the reference's DFS forms.

    Attributes (device tensors over all entries, levels concatenated):
    ``rem`` (remaining budget, or used budget in additive mode), ``start``,
    ``parent`` (global id, -1 for the root), ``dim``/``deg`` (last non-zero
    entry), ``term`` (chain end), ``first_child``/``n_child``; ``level_base``
    (host list) gives the first global id of every level.
    """

    def __init__(self, k: Sequence[float], t: float, mode: int = capi.SMX_MODE_NONZERO):
        dev = device()
        self.mode = mode
        self.k_host = np.ascontiguousarray(np.asarray(k, dtype=np.float64))
        self.d = int(self.k_host.shape[0])
        self.t = float(t)
        self.k = torch.as_tensor(self.k_host, device=dev)
        st = _stream()
        f64, i32, i64 = torch.float64, torch.int32, torch.int64
        rem = torch.tensor([0.0 if mode == capi.SMX_MODE_ADDITIVE else self.t], dtype=f64, device=dev)
        lv = dict(
            rem=[rem],
            start=[torch.zeros(1, dtype=i32, device=dev)],
            parent=[torch.full((1,), -1, dtype=i32, device=dev)],
            dim=[torch.full((1,), -1, dtype=i32, device=dev)],
            deg=[torch.zeros(1, dtype=i32, device=dev)],
            term=[],
            count=[],
            offs=[],
        )
        base = [0]
        while True:
            if len(base) > capi.SMX_MAX_DEPTH + 1:
                raise RuntimeError("index set deeper than %d non-zero entries" % capi.SMX_MAX_DEPTH)
            n = int(lv["rem"][-1].shape[0])
            count = torch.empty(n, dtype=i64, device=dev)
            term = torch.empty(n, dtype=i32, device=dev)
            call("smx_lambda_count", ptr(self.k), self.d, self.t, mode, ptr(lv["rem"][-1]), ptr(lv["start"][-1]), n,
                 ptr(count), ptr(term), st)
            offs = torch.empty(n + 1, dtype=i64, device=dev)
            ws = torch.empty(capi.size("smx_scan_workspace", n), dtype=torch.uint8, device=dev)
            call("smx_scan_i64", ptr(count), ptr(offs), n, ptr(ws), ws.numel(), st)
            lv["term"].append(term)
            lv["count"].append(count)
            lv["offs"].append(offs)
            total = int(offs[n].item())
            if total == 0:
                break
            if base[-1] + n + total >= 2**31:
                raise RuntimeError("index set too large (more than 2^31 entries)")
            ch = dict(rem=torch.empty(total, dtype=f64, device=dev))
            for key in ("start", "parent", "dim", "deg"):
                ch[key] = torch.empty(total, dtype=i32, device=dev)
            call("smx_lambda_expand", ptr(self.k), self.d, self.t, mode, ptr(lv["rem"][-1]), ptr(lv["start"][-1]), n,
                 ptr(offs), base[-1], ptr(ch["rem"]), ptr(ch["start"]), ptr(ch["parent"]), ptr(ch["dim"]),
                 ptr(ch["deg"]), st)
            for key in ch:
                lv[key].append(ch[key])
            base.append(base[-1] + n)
        self.level_base = base + [base[-1] + int(lv["rem"][-1].shape[0])]
        self.n_levels = len(base)
        for key in ("rem", "start", "parent", "dim", "deg", "term", "count"):
            setattr(self, key, torch.cat(lv[key]))
        self.n_child = self.count
        fc = [lv["offs"][i][:-1] + self.level_base[i + 1] for i in range(self.n_levels)]
        self.first_child = torch.cat(fc)
        self.size = int(self.rem.shape[0])
        self._zeta = None
        self._rank = {}

    def level_of(self):
        """Level (number of non-zero entries) of every entry, device int64."""
        lvl = torch.empty(self.size, dtype=torch.int64, device=self.rem.device)
        for n in range(self.n_levels):
            lvl[self.level_base[n] : self.level_base[n + 1]] = n
        return lvl

    def zeta(self):
        """Smolyak coefficient of every entry (``indices.py:121-168``), device int64."""
        if self._zeta is None:
            assert self.mode == capi.SMX_MODE_NONZERO
            z = torch.empty(self.size, dtype=torch.int64, device=self.rem.device)
            flag = torch.zeros(1, dtype=torch.int32, device=self.rem.device)
            call("smx_zeta", ptr(self.k), self.d, ptr(self.rem), None, self.size, ptr(z), ptr(flag), _stream())
            if int(flag.item()) != 0:
                raise RuntimeError("Smolyak coefficient enumeration deeper than %d dimensions" % capi.SMX_MAX_DEPTH)
            self._zeta = z
        return self._zeta

    def rank(self, mode=None):
        """Position of every entry in the reference's DFS emission order, device int64."""
        mode = self.mode if mode is None else mode
        if mode not in self._rank:
            dev = self.rem.device
            st = _stream()
            size = torch.empty(self.size, dtype=torch.int64, device=dev)
            for n in reversed(range(self.n_levels)):
                call("smx_lambda_subtree_sizes", ptr(self.first_child), ptr(self.n_child), self.level_base[n],
                     self.level_base[n + 1], ptr(size), st)
            base = torch.zeros(self.size, dtype=torch.int64, device=dev)
            rank = torch.empty(self.size, dtype=torch.int64, device=dev)
            for n in range(self.n_levels):
                call("smx_lambda_ranks", mode, ptr(self.term), ptr(self.dim), ptr(self.first_child), ptr(self.n_child),
                     ptr(size), self.level_base[n], self.level_base[n + 1], ptr(base), ptr(rank), st)
            self._rank[mode] = rank
        return self._rank[mode]

    def host_tuples(self, order):
        """Sparse multi-index tuples of the entries listed in ``order`` (host)."""
        parent = self.parent.cpu().numpy()
        dim = self.dim.cpu().numpy()
        deg = self.deg.cpu().numpy()
        memo = {}

        def tup(e):
            if e in memo:
                return memo[e]
            if e == 0:
                memo[e] = ()
                return ()
            chain = []
            x = e
            while x > 0 and x not in memo:
                chain.append(x)
                x = int(parent[x])
            out = memo[x] if x in memo else ()
            for y in reversed(chain):
                out = out + ((int(dim[y]), int(deg[y])),)
                memo[y] = out
            return out

        return [tup(int(e)) for e in order]


def indexset(k: Sequence[float], t: float) -> list:
    """Lambda_{k,t} as sparse tuples, in the reference's order (``indices.py:20-69``)."""
    tree = LambdaTree(k, t, capi.SMX_MODE_INDEXSET)
    order = torch.argsort(tree.rank()).cpu().numpy()
    return tree.host_tuples(order)


def indexset_cardinality(k: Sequence[float], t: float) -> int:
    """|Lambda_{k,t}| with the reference's additive test (``indices.py:72-118``)."""
    return LambdaTree(k, t, capi.SMX_MODE_ADDITIVE).size


def smolyak_coefficient(k: Sequence[float], d: int, rem_t: float, parity: int) -> int:
    """Signed count of admissible e in {0,1}^d (``indices.py:121-168``)."""
    dev = device()
    kk = torch.as_tensor(np.asarray(k, dtype=np.float64), device=dev)
    rem = torch.tensor([float(rem_t)], dtype=torch.float64, device=dev)
    par = torch.tensor([int(parity)], dtype=torch.int32, device=dev)
    z = torch.empty(1, dtype=torch.int64, device=dev)
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    call("smx_zeta", ptr(kk), int(d), ptr(rem), ptr(par), 1, ptr(z), ptr(flag), _stream())
    if int(flag.item()):
        raise RuntimeError("Smolyak coefficient enumeration deeper than %d dimensions" % capi.SMX_MAX_DEPTH)
    return int(z.item())


def _prod_degrees(tree: LambdaTree):
    """prod_j (nu_j + 1) of every entry (device int64)."""
    prod = torch.ones(tree.size, dtype=torch.int64, device=tree.rem.device)
    for n in range(1, tree.n_levels):
        b0, b1 = tree.level_base[n], tree.level_base[n + 1]
        prod[b0:b1] = prod[tree.parent[b0:b1].long()] * (tree.deg[b0:b1].long() + 1)
    return prod


def nodeset_cardinality(k: Sequence[float], t: float, nested: bool = False) -> int:
    """Number of interpolation nodes (``indices.py:262-289``)."""
    if nested:
        return indexset_cardinality(k, t)
    tree = LambdaTree(k, t, capi.SMX_MODE_NONZERO)
    z = tree.zeta()
    return int(torch.where(z != 0, _prod_degrees(tree), 0).sum().item())


def non_zero_indices_and_zetas(k: Sequence[float], t: float):
    """Multi-indices with non-zero Smolyak coefficient binned by n, in the
    reference's order (``indices.py:214-259``)."""
    tree = LambdaTree(k, t, capi.SMX_MODE_NONZERO)
    return nonzero_from_tree(tree)


def nonzero_from_tree(tree: LambdaTree):
    z = tree.zeta()
    keep = torch.nonzero(z != 0).flatten()
    order = keep[torch.argsort(tree.rank()[keep])]
    zs = z[order].cpu().numpy()
    nus = tree.host_tuples(order.cpu().numpy())
    n2nus, n2zetas = defaultdict(list), defaultdict(list)
    for nu, zv in zip(nus, zs):
        n2nus[len(nu)].append(nu)
        n2zetas[len(nu)].append(int(zv))
    return n2nus, n2zetas


def find_approximate_threshold(k: Sequence[float], m: int, nested: bool, max_iter: int = 32,
                               accuracy: float = 0.001) -> float:
    """Bracket by factors of 1.2, then bisect; every cardinality is computed on the
    GPU (``indices.py:292-355``)."""
    assert m > 0
    if m == 1:
        return 1
    lo, hi = 1.0, 2.0
    while nodeset_cardinality(k, lo, nested) > m:
        lo, hi = lo / 1.2, lo
    while nodeset_cardinality(k, hi, nested) < m:
        lo, hi = hi, hi * 1.2
    t_c = lo + (hi - lo) / 2.0
    m_c = nodeset_cardinality(k, t_c, nested)
    for _ in range(max_iter):
        if m_c > m:
            hi = t_c
        else:
            lo = t_c
        t_c = lo + (hi - lo) / 2.0
        m_c = nodeset_cardinality(k, t_c, nested)
        if np.abs(m_c - m) / m < accuracy:
            break
    return t_c
