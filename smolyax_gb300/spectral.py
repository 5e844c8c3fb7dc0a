"""Set-up of the mixed-precision (orthogonal-polynomial) form of an interpolant.

The FP64 combination data of a built interpolant (pairs, summands, nodal
values) are converted on the device into coefficients over the index set,
then laid out for the FP32 evaluator of ``csrc/spectral.cu``:

* hot dimensions -- those that occur before another dimension in some
  multi-index; their basis values are tabulated per point in shared memory;
* hot entries    -- multi-indices over hot dimensions only, visited in DFS
  pre-order so that the running product of the path stays in registers;
* cold entries   -- a hot prefix extended by one cold (last) dimension, grouped
  by that dimension so its input column is read once.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi as capi
from ._capi import call, ptr

FAMILIES = {"legendre": 0, "hermite": 1}


class SpectralPlan:
    """Device arrays and the ``smx_spectral`` struct of one interpolant."""

    def __init__(self, ip):
        pl = ip._plan
        tree = ip._tree
        dev = tree.rem.device
        st = capi.stream_ptr(torch.cuda.current_stream())
        c = pl.c
        d, d_out = c.d_in, c.d_out
        self.keep = {}
        T = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)

        # per-dimension family and affine map to the family's variable
        fam, fa, fb = np.zeros(d, np.int32), np.zeros(d), np.zeros(d)
        for j, g in enumerate(ip._node_gen):
            name, a, b = g.spectral_map()
            fam[j], fa[j], fb[j] = FAMILIES[name], a, b
        self.fam = T(fam, torch.int32)
        self.fa64, self.fb64 = T(fa, torch.float64), T(fb, torch.float64)

        # coefficients over Lambda (FP64)
        pdeg_h = pl.keep["pair_deg"].cpu().numpy().astype(np.int64)
        aoff_h = np.concatenate([[0], np.cumsum((pdeg_h + 1) ** 2)[:-1]]) if c.n_pairs else np.zeros(1, np.int64)
        aoff = T(aoff_h, torch.int64)
        A = torch.empty(max(int(((pdeg_h + 1) ** 2).sum()), 1), dtype=torch.float64, device=dev)
        flag = torch.zeros(1, dtype=torch.int32, device=dev)
        call("smx_spectral_pairs", c.n_pairs, ptr(pl.keep["pair_dim"]), ptr(pl.keep["pair_deg"]),
             ptr(pl.keep["pair_voff"]), ptr(aoff), ptr(pl.keep["node"]), ptr(self.fam), ptr(self.fa64),
             ptr(self.fb64), ptr(A), ptr(flag), st)
        if int(flag.item()):
            raise RuntimeError("orthogonal-basis set-up failed (code %d)" % int(flag.item()))
        n_lam = tree.size
        R = c.n_entries
        G = torch.empty(max(R * d_out, 1), dtype=torch.float64, device=dev)
        ids = torch.empty(max(R, 1), dtype=torch.int32, device=dev)
        C = torch.empty(n_lam * d_out, dtype=torch.float64, device=dev)
        call("smx_spectral_coefficients", pl.ref(), ptr(aoff), ptr(A), ptr(tree.first_child), ptr(tree.n_child),
             ptr(tree.dim), ptr(tree.deg), n_lam, ptr(G), ptr(ids), ptr(C), ptr(flag), st)
        if int(flag.item()):
            raise RuntimeError("orthogonal-basis coefficients: multi-index missing from the tree")
        self.C64 = C.view(n_lam, d_out)
        del G, ids, A

        # layout: hot dimensions, hot tape (pre-order), cold groups
        level = tree.level_of()
        parent = tree.parent.long()
        dim = tree.dim.long()
        deg = tree.deg.long()
        nonroot = torch.arange(1, n_lam, device=dev)
        inner = nonroot[parent[nonroot] > 0]  # entries whose parent is not the root
        hot = torch.zeros(d, dtype=torch.bool, device=dev)
        if inner.numel():
            hot[dim[parent[inner]]] = True
        maxdeg = torch.as_tensor(ip._maxdeg, device=dev)
        hot_dims = torch.nonzero(hot).flatten()
        hot_deg = maxdeg[hot_dims]
        hot_soff = torch.zeros_like(hot_deg)
        if hot_dims.numel() > 1:
            hot_soff[1:] = torch.cumsum(hot_deg, 0)[:-1]
        n_hot_slots = int(hot_deg.sum().item()) if hot_dims.numel() else 0
        hot_index = torch.full((d,), -1, dtype=torch.long, device=dev)
        hot_index[hot_dims] = torch.arange(hot_dims.numel(), device=dev)

        is_hot_e = torch.zeros(n_lam, dtype=torch.bool, device=dev)
        is_hot_e[nonroot] = hot[dim[nonroot]]
        hot_e = nonroot[is_hot_e[nonroot]]
        cold_e = nonroot[~is_hot_e[nonroot]]
        # prefix products needed by cold entries: their parents (excluding the root)
        vp_index = torch.zeros(n_lam, dtype=torch.long, device=dev)
        if cold_e.numel():
            par = torch.unique(parent[cold_e])
            par = par[par > 0]
            vp_index[par] = torch.arange(1, par.numel() + 1, device=dev)
            n_vp = int(par.numel()) + 1
        else:
            n_vp = 1
        if n_vp >= 4096:
            raise RuntimeError("too many stored prefixes (%d) for the FP32 evaluator" % n_vp)
        # pre-order of hot entries
        rank = tree.rank(capi.SMX_MODE_PREORDER)
        hot_e = hot_e[torch.argsort(rank[hot_e])]
        depth = level[hot_e]
        max_depth = int(depth.max().item()) if hot_e.numel() else 0
        if max_depth > 8:
            raise RuntimeError("hot multi-indices deeper than 8 are not supported by the FP32 evaluator")
        slot = hot_soff[hot_index[dim[hot_e]]] + deg[hot_e] - 1
        tape = (slot | (depth << 16) | (vp_index[hot_e] << 20)).to(torch.int32)
        # cold entries grouped by (dim, deg)
        if cold_e.numel():
            key = dim[cold_e] * 64 + deg[cold_e]
            cold_e = cold_e[torch.argsort(key, stable=True)]
            cd = dim[cold_e]
            groups, counts = torch.unique_consecutive(cd, return_counts=True)
            cold_off = torch.zeros(groups.numel() + 1, dtype=torch.long, device=dev)
            cold_off[1:] = torch.cumsum(counts, 0)
            gmax = maxdeg[groups]
            cold_ent = (vp_index[parent[cold_e]] | (deg[cold_e] << 24)).to(torch.int32)
        else:
            groups = torch.zeros(0, dtype=torch.long, device=dev)
            cold_off = torch.zeros(1, dtype=torch.long, device=dev)
            gmax = torch.zeros(0, dtype=torch.long, device=dev)
            cold_ent = torch.zeros(0, dtype=torch.int32, device=dev)
        C32 = self.C64.float()
        k = self.keep
        k["hot_dim"] = hot_dims.to(torch.int32).contiguous()
        k["hot_deg"] = hot_deg.to(torch.int32).contiguous()
        k["hot_soff"] = hot_soff.to(torch.int32).contiguous()
        k["tape"] = tape.contiguous()
        k["tape_c"] = C32[hot_e].contiguous()
        k["cold_dim"] = groups.to(torch.int32).contiguous()
        k["cold_gmax"] = gmax.to(torch.int32).contiguous()
        k["cold_off"] = cold_off.to(torch.int32).contiguous()
        k["cold_ent"] = cold_ent.contiguous()
        k["cold_c"] = C32[cold_e].contiguous()
        k["fam_a"] = self.fa64.float().contiguous()
        k["fam_b"] = self.fb64.float().contiguous()
        k["fam"] = self.fam
        k["c0"] = C32[0].contiguous()
        s = capi.SmxSpectral()
        s.d_in, s.d_out = d, d_out
        s.n_hot_slots, s.n_vp, s.n_hot_dims = n_hot_slots, n_vp, int(hot_dims.numel())
        s.n_tape, s.n_cold_groups, s.n_cold = int(hot_e.numel()), int(groups.numel()), int(cold_e.numel())
        s.max_depth = max_depth
        for name in ("hot_dim", "hot_deg", "hot_soff", "tape", "tape_c", "cold_dim", "cold_gmax", "cold_off",
                     "cold_ent", "cold_c", "fam_a", "fam_b", "fam", "c0"):
            t = k[name]
            setattr(s, name, t.data_ptr() if t.numel() else None)
        self.c = s
        self.hot_e, self.cold_e = hot_e, cold_e

    def ref(self):
        import ctypes

        return ctypes.byref(self.c)

    def evaluate(self, x, y):
        """y[P, d_out] (FP32) at x[P, d_in] (FP64, contiguous, on the device)."""
        st = capi.stream_ptr(torch.cuda.current_stream())
        call("smx_spectral_eval", self.ref(), ptr(x), int(x.shape[0]), int(x.shape[1]), ptr(y), st)
        return y
