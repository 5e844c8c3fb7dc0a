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
TC_MIN_DOUT = 16  # from this many outputs on, the tensor-core contraction is used
BLOCKED_TC_TABLES = dict(i32=("tc_td", "tc_row", "tc_chunk", "tc_b", "tc_box"), f32=("tc_tdab",),
                         scalars=("tc_n_td", "tc_n_phi", "tc_n_phi_pad", "tc_n_rows", "tc_max_depth", "tc_n_agen",
                                  "tc_n_chunks", "tc_n_boxes", "tc_lin0", "tc_stages", "tc_td_col", "tc_td_bytes",
                                  "c0"))
MAX_DEGREE = 512  # recurrence tables of the kernels


def _phi_table(fam, z, n):
    """phi_0..phi_n at z (rows), the kernels' three-term recurrence in FP64."""
    out = np.empty((n + 1,) + np.shape(z))
    out[0] = 1.0
    pm1, p = np.zeros_like(z), np.ones_like(z)
    for m in range(n):
        if fam == 0:
            a, b = (2 * m + 1) / (m + 1), m / (m + 1)
        else:
            a, b = np.sqrt(2.0 / (m + 1)), np.sqrt(m / (m + 1))
        pm1, p = p, a * z * p - b * pm1
        out[m + 1] = p
    return out


def basis_change_quadrature(pdim, pdeg, pvoff, node, fam, fa, fb):
    """Per pair, A[m][j] = coefficient of phi_m in the Lagrange polynomial l_j of
    the pair's nodes, by Gauss quadrature (exact for these degrees, no matrix
    inversion): A[m][j] = sum_q w_q l_j(s_q) phi_m(s_q) / h_m."""
    out = []
    for u in range(len(pdeg)):
        g = int(pdeg[u])
        d = int(pdim[u])
        z = fa[d] * node[pvoff[u] : pvoff[u] + g + 1] + fb[d]
        if fam[d] == 0:
            sq, wq = np.polynomial.legendre.leggauss(g + 1)
            h = 2.0 / (2 * np.arange(g + 1) + 1)
        else:
            sq, wq = np.polynomial.hermite.hermgauss(g + 1)
            h = np.full(g + 1, np.sqrt(np.pi))
        bw = 1.0 / np.prod(np.where(np.eye(g + 1, dtype=bool), 1.0, z[:, None] - z[None, :]), axis=1)
        diff = sq[:, None] - z[None, :]
        hit = diff == 0
        with np.errstate(divide="ignore", invalid="ignore"):
            L = bw[None, :] / diff
        with np.errstate(divide="ignore", invalid="ignore"):
            L = L / L.sum(axis=1, keepdims=True)
        rows = np.nonzero(hit.any(axis=1))[0]
        L[rows] = hit[rows].astype(float)
        Phi = _phi_table(int(fam[d]), sq, g)  # [m][q]
        A = (Phi * wq[None, :]) @ L / h[:, None]
        out.append(A.ravel())
    return np.concatenate(out) if out else np.zeros(1)


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
        flag = torch.zeros(1, dtype=torch.int32, device=dev)
        if c.n_pairs and int(pdeg_h.max()) >= MAX_DEGREE:
            raise RuntimeError("pair degree %d exceeds the orthogonal form's limit %d" % (int(pdeg_h.max()),
                                                                                       MAX_DEGREE - 1))
        if c.n_pairs and int(pdeg_h.max()) + 1 > 24:
            # high degrees: inversion-free basis change by Gauss quadrature (host, FP64)
            A = T(basis_change_quadrature(pl.keep["pair_dim"].cpu().numpy(), pdeg_h,
                                          pl.keep["pair_voff"].cpu().numpy(), pl.keep["node"].cpu().numpy(),
                                          fam, fa, fb), torch.float64)
        else:
            A = torch.empty(max(int(((pdeg_h + 1) ** 2).sum()), 1), dtype=torch.float64, device=dev)
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
        nws = capi.size("smx_spectral_coefficients_workspace", pl.ref())
        ws = torch.empty(max(nws, 1), dtype=torch.uint8, device=dev)
        call("smx_spectral_coefficients", pl.ref(), ptr(aoff), ptr(A), ptr(tree.first_child), ptr(tree.n_child),
             ptr(tree.dim), ptr(tree.deg), n_lam, ptr(G), ptr(ids), ptr(C), ptr(flag), ptr(ws), nws, st)
        if int(flag.item()):
            raise RuntimeError("orthogonal-basis coefficients: multi-index missing from the tree")
        self.C64 = C.view(n_lam, d_out)
        del G
        self.A, self.aoff, self.ids = A, aoff, ids  # kept for the adjoint (backward w.r.t. nodal values)

        # layout for the FP32 evaluator (host construction from the device tree)
        tree_np = dict(
            parent=tree.parent.cpu().numpy().astype(np.int64),
            dim=tree.dim.cpu().numpy().astype(np.int64),
            deg=tree.deg.cpu().numpy().astype(np.int64),
            level=tree.level_of().cpu().numpy(),
            rank=tree.rank(capi.SMX_MODE_PREORDER).cpu().numpy(),
            rem=tree.rem.cpu().numpy(),
        )
        C32 = self.C64.float().cpu().numpy()
        lay = build_layout(tree_np, C32, np.asarray(ip._maxdeg), d, d_out, fam, fa, fb)
        self.layout = lay
        k = self.keep
        for name in ("hot_dim", "hot_deg", "hot_soff", "node", "cold", "run", "blk_dims", "blk_run"):
            k[name] = T(lay[name], torch.int32)
        for name in ("node_c", "coef", "cold_ab", "blk_ab"):
            k[name] = T(lay[name], torch.float32)
        k["fam_a"] = self.fa64.float().contiguous()
        k["fam_b"] = self.fb64.float().contiguous()
        k["fam"] = self.fam
        k["c0"] = T(C32[0], torch.float32)
        s = capi.SmxSpectral()
        s.d_in, s.d_out = d, d_out
        for name in ("dstride", "row", "n_hb", "n_vp", "n_hot_dims", "n_nodes", "n_cold_groups", "max_depth",
                     "n_cold_blocks"):
            setattr(s, name, int(lay[name]))
        for i in range(5):
            s.node_seg[i] = int(lay["node_seg"][i])
            s.cold_seg[i] = int(lay["cold_seg"][i])
            s.block_seg[i] = int(lay["block_seg"][i])
        for name in ("hot_dim", "hot_deg", "hot_soff", "node", "node_c", "cold", "cold_ab", "run", "coef", "fam_a",
                     "fam_b", "fam", "c0", "blk_dims", "blk_run", "blk_ab"):
            t = k[name]
            setattr(s, name, t.data_ptr() if t.numel() else None)
        self.c = s
        self.tc = None
        self._bwd = None
        self._fwd_args = (tree_np, C32, np.asarray(ip._maxdeg), fam, fa, fb, T, st)
        self.plan = pl
        stream_fits = (lay["row"] + 4 * (1 if d_out == 1 else 4) * 2) * 128 * 4 <= 220 * 1024
        if d_out >= TC_MIN_DOUT or not stream_fits:
            self._build_tc(*self._fwd_args)
        self.memory_limit = ip._memory_limit
        self._f64 = None
        self.blocked = None
        self.blocked_tc = None
        if d_out == 1 and self.tc is None:
            self._build_blocked(tree_np, C32[:, 0], np.asarray(ip._maxdeg), d, fam, fa, fb, T)

    def _build_tc(self, tr, C32, maxdeg, fam, fa, fb, T, st):
        """Operands of the tensor-core contraction: tape over all non-root entries
        (pre-order), coefficient matrix B = C^T split into TF32 hi/lo."""
        self.tree_np, self.maxdeg = tr, maxdeg
        tp = build_tape(tr, maxdeg)
        if tp is None:
            return  # the FP32 stream evaluator serves this plan
        dims, dmax, dsoff, n_slots, tape, ent = (tp[key] for key in ("dims", "dmax", "dsoff", "n_slots", "tape", "ent"))
        K = int(ent.size)
        ldk = _round32(max(K, 1))  # 128-byte rows: whole cache lines per TMA row of B
        d_out = C32.shape[1]
        B = np.zeros((d_out, ldk), dtype=np.float32)
        B[:, :K] = C32[ent[::-1]].T  # the panel stores the entries in reversed pre-order
        dev = self.fam.device
        Bd = T(B, torch.float32)
        Bh, Bl = torch.empty_like(Bd), torch.empty_like(Bd)
        call("smx_split_tf32", ptr(Bd), d_out, ldk, ldk, ptr(Bh), ptr(Bl), ldk, st)
        self.tc = dict(dims=T(dims, torch.int32), dmax=T(dmax, torch.int32), dsoff=T(dsoff, torch.int32),
                       n_slots=n_slots, tape=T(tape, torch.int32), K=K, ldk=ldk, Bh=Bh, Bl=Bl, Bd=Bd,
                       bias=self.keep["c0"], err=torch.zeros(1, dtype=torch.int32, device=dev),
                       ent=torch.as_tensor(ent, device=dev),
                       # tape positions of the depth-1 entries: where independent segments may start
                       lvl1=np.nonzero(tr["level"][ent] == 1)[0],
                       sms=torch.cuda.get_device_properties(dev).multi_processor_count)

    def _build_blocked(self, tr, c, maxdeg, d, fam, fa, fb, T):
        """Tables of the blocked evaluator (one output), if the plan fits it."""
        from .blocked import build_blocked

        self._blocked_args = (tr, c, maxdeg, d, fam, fa, fb, T)
        lay = build_blocked(tr, c, maxdeg, d, fam, fa, fb)
        if lay is None:
            return
        kb = {}
        for name in ("hot_dim", "hot_deg", "hot_soff", "node", "vc", "hot_ent", "grp", "warp_off", "items"):
            kb[name] = T(lay[name], torch.int32)
        for name in ("grp_ab", "W"):
            kb[name] = T(lay[name], torch.float32)
        b = capi.SmxBlocked()
        for name in ("d_in", "n_hs", "k_c", "n_hot_dims", "n_nodes", "n_groups", "n_items"):
            setattr(b, name, int(lay[name]))
        b.c0 = float(lay["c0"])
        for name, t in kb.items():
            setattr(b, name, t.data_ptr() if t.numel() else None)
        b.fa, b.fb, b.fam = (self.keep[k].data_ptr() for k in ("fam_a", "fam_b", "fam"))
        b.n_ent = int(np.asarray(lay["hot_ent"]).size)
        b.n_w = int(np.asarray(lay["W"]).size) // 4
        self.blocked = b
        self.blocked_keep = kb
        self.blocked_layout = lay
        self._build_blocked_tc(tr, c, maxdeg, fam, fa, fb, T)

    def _build_blocked_tc(self, tr, c, maxdeg, fam, fa, fb, T):
        """Tables of the tensor-core blocked evaluator (library builder), if the plan fits it."""
        self.blocked_tc = None
        lay = capi.host_layout("blocked_tc", tr, np.asarray(c, dtype=np.float32).reshape(-1, 1), 1, maxdeg, fam, fa,
                               fb, **BLOCKED_TC_TABLES)
        if lay is None:
            return
        kt = dict(td=T(lay["tc_td"], torch.int32), tdab=T(lay["tc_tdab"], torch.float32),
                  row=T(lay["tc_row"], torch.int32), bimg=T(lay["tc_b"], torch.int32),
                  box=T(lay["tc_box"], torch.int32), err=T(np.zeros(1, np.int32), torch.int32))
        chunk = np.ascontiguousarray(lay["tc_chunk"], dtype=np.int32)
        b = capi.SmxBlockedTc()
        b.d_in = int(np.asarray(maxdeg).shape[0])
        for name in ("n_td", "n_phi", "n_phi_pad", "n_rows", "max_depth", "n_agen", "n_chunks", "n_boxes", "lin0",
                     "stages", "td_col", "td_bytes"):
            setattr(b, name, int(lay["tc_" + name]))
        b.c0 = float(lay["c0"])
        for name in ("td", "tdab", "row", "bimg", "box", "err"):
            setattr(b, name, kt[name].data_ptr() if kt[name].numel() else None)
        b.chunk = chunk.ctypes.data
        self.blocked_tc = b
        self.blocked_tc_keep = (kt, chunk)

    def ref(self):
        import ctypes

        return ctypes.byref(self.c)

    # ------------------------------------------------------------------ backward
    def _backward_ops(self):
        """Tape operands (built as for the forward tensor-core path) plus the
        coefficient rows C[K x ldo] in the panel's reversed order, TF32 hi/lo."""
        if self._bwd is None:
            fwd_tc = self.tc
            self._build_tc(*self._fwd_args)
            ops = self.tc
            self.tc = fwd_tc
            if ops is None:
                raise RuntimeError("backward needs Smolyak index depth <= 8 (register product stack)")
            T = self._fwd_args[6]
            st = self._fwd_args[7]
            C32 = self._fwd_args[1]
            K = ops["K"]
            d_out = C32.shape[1]
            ldo = _round4(d_out)
            ent = ops["ent"].cpu().numpy()
            rows = np.zeros((max(K, 1), ldo), dtype=np.float32)
            rows[:K, :d_out] = C32[ent[::-1]]
            Rd = T(rows, torch.float32)
            Rh, Rl = torch.empty_like(Rd), torch.empty_like(Rd)
            call("smx_split_tf32", ptr(Rd), rows.shape[0], ldo, ldo, ptr(Rh), ptr(Rl), ldo, st)
            ops.update(Rh=Rh, Rl=Rl, ldo=ldo)
            # tape segments of the gradient walk: fixed per plan (a point's dL/dx
            # does not depend on the batch it comes in)
            want = vjp_segment_count(K, ops["lvl1"].size)
            if want > 1:
                b = T(segment_bounds(ops["lvl1"], K, want), torch.int32)
                ops["vjp_seg"] = (b, int(b.numel()) - 1)
            else:
                ops["vjp_seg"] = (None, 1)
            self._bwd = ops
        return self._bwd

    def vjp(self, x, g, need_x=True, need_coef=True, check=True):
        """Vector-Jacobian products of y = c0 + A(x) C at cotangent g [P, d_out]:
        returns (dL/dx [P, d_in] FP64 or None, dL/dC [n_lambda, d_out] FP64 or None)."""
        ops = self._backward_ops()
        st = capi.stream_ptr(torch.cuda.current_stream())
        k = self.keep
        dev = x.device
        P, d = int(x.shape[0]), int(x.shape[1])
        d_out = int(g.shape[1])
        K, ldk, ldo = ops["K"], ops["ldk"], ops["ldo"]
        nd = int(ops["dims"].numel())
        common = (nd, ptr(ops["dims"]), ptr(ops["dmax"]), ptr(ops["dsoff"]), ops["n_slots"], ptr(ops["tape"]), K,
                  ptr(k["fam_a"]), ptr(k["fam_b"]), ptr(k["fam"]))
        seg, n_seg = ops["vjp_seg"]
        walk = (nd, ptr(ops["dims"]), ptr(ops["dmax"]), ptr(ops["dsoff"]), ops["n_slots"], ptr(ops["tape"]), K,
                ptr(seg), n_seg, ptr(k["fam_a"]), ptr(k["fam_b"]), ptr(k["fam"]))
        g32 = torch.zeros(P, ldo, dtype=torch.float32, device=dev)
        g32[:, :d_out] = g.float()
        gh, gl = torch.empty_like(g32), torch.empty_like(g32)
        call("smx_split_tf32", ptr(g32), P, ldo, ldo, ptr(gh), ptr(gl), ldo, st)
        err = ops["err"]
        dx = dC = None
        step = max(128, int(self.memory_limit * 1024**3 // (8 * ldk)) // 128 * 128)
        if need_x:
            dx = torch.zeros(P, d, dtype=torch.float64, device=dev)
            ldg = _round32(K)  # 128-byte rows
            G = torch.empty(min(step, P), ldg, dtype=torch.float32, device=dev)
            nws = capi.size("smx_spectral_vjp_x_workspace", ops["n_slots"], n_seg, min(step, P))
            ws = torch.empty(max(nws, 1), dtype=torch.uint8, device=dev)
            for p0 in range(0, P, step):
                p1 = min(P, p0 + step)
                call("smx_gemm_tf32x3", ptr(gh[p0:p1]), ptr(gl[p0:p1]), ldo, ptr(ops["Rh"]), ptr(ops["Rl"]), ldo,
                     p1 - p0, K, ldo, ptr(G), ldg, None, 0, ptr(err), st)
                call("smx_spectral_vjp_x", *walk, ptr(x[p0:p1]), p1 - p0, d, ptr(G), ldg, ptr(dx[p0:p1]), d,
                     ptr(ws), nws, st)
        if need_coef:
            ldp = _round32(min(step, P))  # 128-byte rows
            ATh = torch.empty(K, ldp, dtype=torch.float32, device=dev)
            ATl = torch.empty_like(ATh)
            gT = torch.zeros(ldo, ldp, dtype=torch.float32, device=dev)
            gTh, gTl = torch.empty_like(gT), torch.empty_like(gT)
            dCrev = torch.zeros(K, d_out, dtype=torch.float32, device=dev)
            nws = capi.size("smx_spectral_panel_t_workspace", ops["n_slots"], min(step, P))
            ws = torch.empty(max(nws, 1), dtype=torch.uint8, device=dev)
            # the [K x d_out] product has few tiles and a long contraction over the
            # points: split the contraction so that the slices fill the SMs
            tiles = -(-K // 128) * -(-d_out // 128)
            splits = max(1, min(64, (2 * ops["sms"]) // tiles))
            nsk = capi.size("smx_gemm_tf32x3_splitk_workspace", K, d_out, min(step, P), splits)
            wsk = torch.empty(max(nsk, 1), dtype=torch.uint8, device=dev)
            for i, p0 in enumerate(range(0, P, step)):
                p1 = min(P, p0 + step)
                n = p1 - p0
                # the contraction runs over the chunk's n points: the columns past n
                # are outside the operands' tensor maps and need no zeros
                call("smx_spectral_panel_t_tf32", *common, ptr(x[p0:p1]), n, d, ptr(ATh), ptr(ATl), ldp, ptr(ws), nws,
                     st)
                gT[:, :n] = g32[p0:p1].t()
                call("smx_split_tf32", ptr(gT), ldo, n, ldp, ptr(gTh), ptr(gTl), ldp, st)
                call("smx_gemm_tf32x3_splitk", ptr(ATh), ptr(ATl), ldp, ptr(gTh), ptr(gTl), ldp, K, d_out, n,
                     ptr(dCrev), d_out, None, 1 if i else 0, splits, ptr(wsk), nsk, ptr(err), st)
            n_lam = int(self.C64.shape[0])
            dC = torch.zeros(n_lam, d_out, dtype=torch.float64, device=dev)
            ent = ops["ent"]
            dC[ent.flip(0)] = dCrev.double()
            dC[0] = g.double().sum(0)
        if check and int(err.item()):
            raise RuntimeError("tensor-core contraction reported a pipeline timeout")
        return dx, dC

    def coefficient_adjoint(self, dC):
        """dL/d(plan rows F64) [n_entries, d_out] from dL/dC (FP64 adjoint transform)."""
        pl = self.plan
        R, d_out = pl.c.n_entries, pl.c.d_out
        Fbar = torch.zeros(max(R, 1), d_out, dtype=torch.float64, device=dC.device)
        st = capi.stream_ptr(torch.cuda.current_stream())
        call("smx_spectral_coefficients_adjoint", pl.ref(), ptr(self.aoff), ptr(self.A), ptr(self.ids),
             ptr(dC.contiguous()), ptr(Fbar), st)
        return Fbar[:R]

    def evaluate(self, x, y, mode="tf32x3"):
        """y[P, d_out] (FP32) at x[P, d_in] (FP64, contiguous, on the device).
        ``mode="bf16x3"`` runs the tensor-core contraction with split-BF16
        operands (plans with the tensor-core form only).  ``mode="blocked_tc"``
        evaluates a one-output plan with the tensor-core blocked evaluator
        (``csrc/blocked_tc.cu``: ~2.5x smaller error than the blocked
        evaluator, ~1.6x its time at d_in = 1000)."""
        st = capi.stream_ptr(torch.cuda.current_stream())
        if mode == "bf16x3":
            if self.tc is None:
                raise ValueError("bf16x3 needs the tensor-core form of the plan (16 or more outputs)")
            return self._evaluate_tc(x, y, st, bf16=True)
        if self.tc is not None:
            return self._evaluate_tc(x, y, st)
        if self.blocked is not None:
            import ctypes

            P = int(x.shape[0])
            if mode == "blocked_tc":
                if self.blocked_tc is None:
                    raise ValueError("the plan is outside the tensor-core blocked evaluator's limits")
                ref = ctypes.byref(self.blocked_tc)
                if not capi.size("smx_blocked_tc_supported", ref, ptr(x), int(x.shape[1])):
                    raise ValueError("the tensor-core blocked evaluator needs x 16-byte aligned with an even row pitch")
                call("smx_blocked_tc_eval", ref, ptr(x), P, int(x.shape[1]), ptr(y), st)
                return y
            nws = capi.size("smx_blocked_eval_workspace", ctypes.byref(self.blocked), P)
            ws = torch.empty(max(nws, 1), dtype=torch.uint8, device=x.device)
            call("smx_blocked_eval", ctypes.byref(self.blocked), ptr(x), P, int(x.shape[1]), ptr(y), ptr(ws), nws, st)
            return y
        call("smx_spectral_eval", self.ref(), ptr(x), int(x.shape[0]), int(x.shape[1]), ptr(y), st)
        return y

    def fp64_form(self):
        """FP64 tables of the orthogonal form for ``csrc/spectral64.cu``, built on
        first use from the same tree and the FP64 coefficients; None where that
        evaluator does not apply (hot nodes deeper than 8, or a per-point row
        beyond shared memory)."""
        if self._f64 is None:
            self._f64 = False
            tr, _, maxdeg, fam, fa, fb, T, _ = self._fwd_args
            d = int(self.c.d_in)
            lay = build_layout64(tr, self.C64.cpu().numpy(), maxdeg, d, fam, fa, fb)
            row = int(lay["row"])
            DO = 1 if lay["d_out"] == 1 else 4
            if (row + 4 * DO) * 64 * 8 <= 227 * 1024 and int(lay["max_depth"]) <= 8:
                k = {}
                for name in ("hot_dim", "hot_deg", "hot_soff", "node", "cold", "run"):
                    k[name] = T(lay[name], torch.int32)
                for name in ("node_c", "cold_ab", "terms", "coef"):
                    k[name] = T(lay[name], torch.float64)
                k["c0"] = self.C64[0].contiguous()
                st = capi.SmxSpectral64()
                st.d_in, st.row = d, row
                for name in ("d_out", "dstride", "n_hb", "n_vp", "n_hot_dims", "n_nodes", "n_cold_groups", "max_depth",
                             "n_terms"):
                    setattr(st, name, int(lay[name]))
                for i in range(5):
                    st.node_seg[i] = int(lay["node_seg"][i])
                    st.cold_seg[i] = int(lay["cold_seg"][i])
                for name, t in k.items():
                    setattr(st, name, t.data_ptr() if t.numel() else None)
                st.fam_a, st.fam_b, st.fam = self.fa64.data_ptr(), self.fb64.data_ptr(), self.fam.data_ptr()
                self._f64 = (st, k)
        return self._f64 or None

    def evaluate64(self, x, y):
        """y[P, d_out] (FP64, contiguous) at x[P, d_in] (FP64, rows contiguous, on
        the device) through the FP64 evaluator of the orthogonal form."""
        import ctypes

        form = self.fp64_form()
        if form is None:
            raise ValueError("the plan has no FP64 orthogonal form (a per-point row within shared memory)")
        if x.dim() != 2 or (x.shape[0] > 1 and x.stride(1) != 1):
            x = x.contiguous()
        ldx = int(x.stride(0)) if x.shape[0] > 1 else int(x.shape[1])  # a one-row tensor may carry any row stride
        call("smx_spectral_eval64", ctypes.byref(form[0]), ptr(x), int(x.shape[0]), ldx, ptr(y),
             capi.stream_ptr(torch.cuda.current_stream()))
        return y

    def _tc_step(self, P):
        """Points per panel chunk (the hi/lo panel of one chunk fits the memory limit)."""
        step = max(128, int(self.memory_limit * 1024**3 // (8 * ((self.tc["K"] + 31) // 32 * 32))) // 128 * 128)
        return max(1, min(step, P))

    def tc_splits(self):
        """K slices of the forward contraction (``smx_gemm_tf32x3_splits`` for a
        full panel chunk): a plan constant, so a point's value does not depend
        on the batch it arrives in."""
        if "splits" not in self.tc:
            self.tc["splits"] = capi.size("smx_gemm_tf32x3_splits", self._tc_step(1 << 40),
                                          int(self.tc["Bd"].shape[0]), self.tc["K"])
        return self.tc["splits"]

    def tc_chunks(self, P):
        """Number of panel chunks (each one panel and one GEMM launch) for P points."""
        return -(-int(P) // self._tc_step(P)) if P else 0

    def tc_launches(self, P):
        """Kernel launches of one tensor-core evaluation of P points: per chunk the
        panel (plus its basis-row kernel when the rows go to global scratch) and
        the GEMM."""
        scratch = capi.size("smx_spectral_panel_workspace", self.tc["n_slots"], 1) > 0
        return self.tc_chunks(P) * ((3 if scratch else 2) + (1 if self.tc_splits() > 1 else 0))

    def _segments(self, n):
        """Tape segments of one panel launch over n points (see segment_bounds).
        Returns (bounds on the device or None, count)."""
        tc = self.tc
        want = segment_count(tc["K"], tc["lvl1"].size, n, tc["sms"])
        if want <= 1:
            return None, 1
        cache = tc.setdefault("segs", {})
        if want not in cache:
            cache[want] = torch.as_tensor(segment_bounds(tc["lvl1"], tc["K"], want), device=tc["tape"].device)
        t = cache[want]
        return t, int(t.numel()) - 1

    def _bf16_operands(self):
        """Coefficient matrix B split to BF16 hi/lo (built on first use), rows
        padded to 64 entries (128 bytes)."""
        tc = self.tc
        if "Bh16" not in tc:
            d_out, K = int(tc["Bd"].shape[0]), tc["K"]
            ld16 = (K + 63) // 64 * 64
            Bh = torch.zeros(d_out, ld16, dtype=torch.bfloat16, device=tc["Bd"].device)
            Bl = torch.zeros_like(Bh)
            call("smx_split_bf16", ptr(tc["Bd"]), d_out, K, tc["ldk"], ptr(Bh), ptr(Bl), ld16,
                 capi.stream_ptr(torch.cuda.current_stream()))
            tc.update(Bh16=Bh, Bl16=Bl, ld16=ld16)
        return tc["Bh16"], tc["Bl16"], tc["ld16"]

    def _evaluate_tc(self, x, y, st, bf16=False):
        """Tensor-core path: basis-product panel (TF32 or BF16 hi/lo) in chunks
        of points, each contracted with the coefficient matrix by the tcgen05
        kernel."""
        tc = self.tc
        k = self.keep
        P, d = int(x.shape[0]), int(x.shape[1])
        d_out = int(y.shape[1])
        if bf16:
            Bh, Bl, ld16 = self._bf16_operands()
            step = self._tc_step(P)
            lda = (tc["K"] + 63) // 64 * 64  # 128-byte panel rows
            Ah = torch.empty(step, lda, dtype=torch.bfloat16, device=x.device)
            Al = torch.empty_like(Ah)
            for p0 in range(0, P, step):
                p1 = min(P, p0 + step)
                nws = capi.size("smx_spectral_panel_workspace", tc["n_slots"], p1 - p0)
                ws = torch.empty(max(nws, 1), dtype=torch.uint8, device=x.device)
                seg, n_seg = self._segments(p1 - p0)
                call("smx_spectral_panel_bf16", int(tc["dims"].numel()), ptr(tc["dims"]), ptr(tc["dmax"]),
                     ptr(tc["dsoff"]), tc["n_slots"], ptr(tc["tape"]), tc["K"], ptr(seg), n_seg, ptr(k["fam_a"]),
                     ptr(k["fam_b"]), ptr(k["fam"]), ptr(x[p0:p1]), p1 - p0, d, ptr(Ah), ptr(Al), lda, ptr(ws), nws,
                     st)
                call("smx_gemm_bf16x3", ptr(Ah), ptr(Al), lda, ptr(Bh), ptr(Bl), ld16, p1 - p0, d_out, tc["K"],
                     ptr(y[p0:p1]), d_out, ptr(tc["bias"]), 0, ptr(tc["err"]), st)
            return y
        ldk = tc["ldk"]
        step = self._tc_step(P)
        lda = (tc["K"] + 31) // 32 * 32  # 128-byte panel rows
        Ah = torch.empty(step, lda, dtype=torch.float32, device=x.device)
        Al = torch.empty_like(Ah)
        splits = self.tc_splits()
        if splits > 1:
            nsk = capi.size("smx_gemm_tf32x3_splitk_workspace", step, d_out, tc["K"], splits)
            skws = torch.empty(max(nsk, 1), dtype=torch.uint8, device=x.device)
        for p0 in range(0, P, step):
            p1 = min(P, p0 + step)
            nws = capi.size("smx_spectral_panel_workspace", tc["n_slots"], p1 - p0)
            ws = torch.empty(max(nws, 1), dtype=torch.uint8, device=x.device)
            seg, n_seg = self._segments(p1 - p0)
            call("smx_spectral_panel_tf32", int(tc["dims"].numel()), ptr(tc["dims"]), ptr(tc["dmax"]),
                 ptr(tc["dsoff"]), tc["n_slots"], ptr(tc["tape"]), tc["K"], ptr(seg), n_seg, ptr(k["fam_a"]),
                 ptr(k["fam_b"]), ptr(k["fam"]), ptr(x[p0:p1]), p1 - p0, d, ptr(Ah), ptr(Al), lda, ptr(ws), nws, st)
            if splits > 1:
                call("smx_gemm_tf32x3_splitk", ptr(Ah), ptr(Al), lda, ptr(tc["Bh"]), ptr(tc["Bl"]), ldk, p1 - p0,
                     d_out, tc["K"], ptr(y[p0:p1]), d_out, ptr(tc["bias"]), 0, splits, ptr(skws), nsk, ptr(tc["err"]),
                     st)
            else:
                call("smx_gemm_tf32x3", ptr(Ah), ptr(Al), lda, ptr(tc["Bh"]), ptr(tc["Bl"]), ldk, p1 - p0, d_out,
                     tc["K"], ptr(y[p0:p1]), d_out, ptr(tc["bias"]), 0, ptr(tc["err"]), st)
        return y


def build_tape(tr, maxdeg):
    """Tape of the tensor-core panel: the non-root entries in DFS pre-order,
    word = basis slot | depth << 16, the slots of dimension j (max degree
    m_j > 0) being dsoff[j] .. dsoff[j] + m_j - 1.  None when an entry is
    deeper than 8 (the panel's register product stack)."""
    maxdeg = np.asarray(maxdeg)
    if int(tr["level"].max()) > 8:
        return None
    dims = np.nonzero(maxdeg > 0)[0]
    dmax = maxdeg[dims]
    dsoff = np.concatenate([[0], np.cumsum(dmax)[:-1]]) if dims.size else np.zeros(0, np.int64)
    idx = np.full(maxdeg.shape[0], -1, dtype=np.int64)
    idx[dims] = np.arange(dims.size)
    n = tr["parent"].shape[0]
    ent = np.arange(1, n)
    ent = ent[np.argsort(tr["rank"][ent], kind="stable")]
    slot = dsoff[idx[tr["dim"][ent]]] + tr["deg"][ent] - 1
    tape = (slot | (tr["level"][ent] << 16)).astype(np.int32)
    return dict(dims=dims, dmax=dmax, dsoff=dsoff, n_slots=int(dmax.sum()), tape=tape, ent=ent,
                lvl1=np.nonzero(tr["level"][ent] == 1)[0])


def segment_count(K, n_lvl1, n_points, sms):
    """Segments per panel launch: enough (segment, 128-point block) blocks for
    ~12 per SM, at most 32 segments, segments of >= 256 entries on average, and
    no more than there are depth-1 entries to start them."""
    n_pb = max(-(-int(n_points) // 128), 1)
    return max(1, min(32, -(-12 * int(sms) // n_pb), int(K) // 256, int(n_lvl1)))


def vjp_segment_count(K, n_lvl1):
    """Tape segments of the gradient walk: one per 4096 tape entries (at most
    32 and the number of depth-1 entries), fixed per plan."""
    return max(1, min(32, int(K) // 4096, int(n_lvl1)))


def segment_bounds(lvl1, K, want):
    """Segment bounds [0, ..., K] (int32) near equal splits of the tape: every
    bound but the last is the tape position of a depth-1 entry, so that each
    segment holds whole subtrees (lvl1: sorted positions, lvl1[0] = 0)."""
    lvl1 = np.asarray(lvl1)
    targets = (np.arange(1, want) * int(K)) // want
    b = lvl1[np.minimum(np.searchsorted(lvl1, targets), lvl1.size - 1)]
    return np.unique(np.concatenate([[0], b, [int(K)]])).astype(np.int32)


def _round4(v):
    return (int(v) + 3) // 4 * 4


def _round32(v):
    return (int(v) + 31) // 32 * 32


class _Runs:
    """Accumulates runs (4-aligned slot ranges with contiguous coefficients)."""

    def __init__(self, dstride):
        self.dstride = dstride
        self.tab = []
        self.coef = []
        self.ncoef = 0

    def add(self, slots, coefs, max_gap=4, degree=0, max_len=32):
        """slots: increasing row slots; coefs: [len(slots), d_out]. Returns (r0, r1).
        A run spans at most max_len slots: the evaluator sums each run in plain
        FP32 and adds the run sums with compensation."""
        r0 = len(self.tab)
        i = 0
        n = len(slots)
        while i < n:
            j = i + 1
            a0 = int(slots[i]) & ~3
            while j < n and slots[j] - slots[j - 1] <= max_gap and slots[j] - a0 < max_len:
                j += 1
            length = _round4(int(slots[j - 1]) + 1 - a0)
            blk = np.zeros((length, self.dstride), dtype=np.float32)
            blk[np.asarray(slots[i:j]) - a0, : coefs.shape[1]] = coefs[i:j]
            self.tab.append((a0, length, self.ncoef, degree))
            self.coef.append(blk.ravel())
            self.ncoef += blk.size
            i = j
        return r0, len(self.tab)


def _layout_front(tr, maxdeg, d):
    """The structure shared by the per-point layouts (FP32 and FP64): hot
    dimensions and their basis slots, hot nodes in DFS pre-order, the prefix
    slots of the cold entries' parents (by remaining budget, descending: the
    prefixes admissible for a cold pair are then (mostly) a leading range), and
    each node's hot leaf children sorted by slot."""
    parent, dim, deg, level, rank, rem = (tr[key] for key in ("parent", "dim", "deg", "level", "rank", "rem"))
    n = parent.shape[0]
    nonroot = np.arange(1, n)
    hot = np.zeros(d, dtype=bool)
    inner = nonroot[parent[nonroot] > 0]
    hot[dim[parent[inner]]] = True
    hot_dims = np.nonzero(hot)[0]
    hot_deg = maxdeg[hot_dims].astype(np.int64)
    hot_soff = np.concatenate([[0], np.cumsum(hot_deg)[:-1]]).astype(np.int64) if hot_dims.size else np.zeros(0, np.int64)
    n_hb = int(hot_deg.sum())
    hot_index = np.full(d, -1, dtype=np.int64)
    hot_index[hot_dims] = np.arange(hot_dims.size)
    is_hot = np.zeros(n, dtype=bool)
    is_hot[0] = True
    is_hot[nonroot] = hot[dim[nonroot]]
    cold_e = nonroot[~is_hot[nonroot]]
    hot_e = nonroot[is_hot[nonroot]]
    slot = np.full(n, -1, dtype=np.int64)
    slot[hot_e] = hot_soff[hot_index[dim[hot_e]]] + deg[hot_e] - 1
    has_hot_child = np.zeros(n, dtype=bool)
    has_hot_child[parent[hot_e]] = True
    has_cold_child = np.zeros(n, dtype=bool)
    has_cold_child[parent[cold_e]] = True
    node_mask = is_hot & (has_hot_child | has_cold_child)
    node_mask[0] = True
    nodes = np.nonzero(node_mask)[0]
    nodes = nodes[np.argsort(rank[nodes], kind="stable")]
    S = np.nonzero(has_cold_child)[0]
    S = S[S != 0]
    S = S[np.argsort(-rem[S], kind="stable")]
    vp_row = np.full(n, -1, dtype=np.int64)
    vp_row[0] = n_hb
    vp_row[S] = n_hb + 1 + np.arange(S.size)
    leaf_e = hot_e[~node_mask[hot_e]]
    leaf_e = leaf_e[np.lexsort((slot[leaf_e], parent[leaf_e]))]
    lp = parent[leaf_e]
    return dict(parent=parent, dim=dim, deg=deg, level=level, hot_dims=hot_dims, hot_deg=hot_deg, hot_soff=hot_soff,
                n_hb=n_hb, cold_e=cold_e, slot=slot, nodes=nodes, vp_row=vp_row, n_vp=1 + S.size, leaf_e=leaf_e,
                starts=np.searchsorted(lp, nodes, side="left"), ends=np.searchsorted(lp, nodes, side="right"),
                max_depth=int(level[nodes].max()) if nodes.size else 0)


def _cuts(cost, allowed, nseg):
    """Segment boundaries: boundary k is the allowed index whose cumulative
    cost is nearest k/nseg of the total (the first such, not before the
    previous boundary)."""
    tot = float(np.sum(cost))
    cum = np.concatenate([[0.0], np.cumsum(cost)])
    out = [0]
    for k in range(1, nseg):
        want = tot * k / nseg
        cand = [a for a in allowed if a >= out[-1]]
        out.append(min(cand, key=lambda a: abs(cum[a] - want)) if cand else out[-1])
    out.append(len(cost))
    return out


def build_layout(tr, C, maxdeg, d, d_out, fam, fa, fb, nseg=4):
    """Layout of the FP32 per-point evaluator (see ``csrc/spectral.cu``) from
    the index-set tree (host arrays: parent, dim, deg, level, pre-order rank,
    remaining budget) and the FP32 coefficients C[entry, d_out]; fam/fa/fb are
    the per-dimension polynomial family and affine map to its variable."""
    fr = _layout_front(tr, maxdeg, d)
    parent, dim, deg, level = fr["parent"], fr["dim"], fr["deg"], fr["level"]
    hot_dims, hot_deg, hot_soff, n_hb = fr["hot_dims"], fr["hot_deg"], fr["hot_soff"], fr["n_hb"]
    cold_e, slot, nodes, vp_row, n_vp = fr["cold_e"], fr["slot"], fr["nodes"], fr["vp_row"], fr["n_vp"]
    leaf_e, starts, ends, max_depth = fr["leaf_e"], fr["starts"], fr["ends"], fr["max_depth"]
    dstride = 1 if d_out == 1 else _round4(d_out)
    row = _round4(n_hb + n_vp)
    while row % 32 != 4:
        row += 4
    runs = _Runs(dstride)
    node_tab = np.zeros((nodes.size, 4), dtype=np.int64)
    node_c = np.zeros((nodes.size, dstride), dtype=np.float32)
    cost_nodes = np.zeros(nodes.size)
    for i, e in enumerate(nodes):
        le = leaf_e[starts[i] : ends[i]]
        r0, r1 = runs.add(slot[le], C[le])
        sl = int(slot[e]) if e != 0 else 0
        node_tab[i] = (sl | (int(level[e]) << 16), int(vp_row[e]) if e != 0 and vp_row[e] >= 0 else -1, r0, r1)
        if e != 0:  # the root's coefficient is added once, as c0, by the evaluator
            node_c[i, :d_out] = C[e]
        cost_nodes[i] = 12 + sum(t[1] for t in runs.tab[r0:r1]) / 4.0 * (1 + d_out)
    # cold dimensions: entries sorted by (dim, deg, prefix slot)
    ce = cold_e[np.lexsort((vp_row[parent[cold_e]], deg[cold_e], dim[cold_e]))] if cold_e.size else cold_e
    bounds = []
    i = 0
    while i < ce.size:
        j = i
        while j < ce.size and dim[ce[j]] == dim[ce[i]]:
            j += 1
        bounds.append((i, j))
        i = j
    simple = [b for b in bounds if d_out == 1 and np.all(deg[ce[b[0] : b[1]]] == 1)]
    general = [b for b in bounds if not (d_out == 1 and np.all(deg[ce[b[0] : b[1]]] == 1))]
    alpha0 = np.where(np.asarray(fam) == 0, 1.0, np.sqrt(2.0))
    # blocks of 4 degree-1 cold dimensions sharing one run of prefix slots
    blk_dims, blk_run, blk_ab, cost_blk = [], [], [], []
    for q in range(0, len(simple), 4):
        part = simple[q : q + 4]
        dims4 = [int(dim[ce[b0]]) for b0, _ in part]
        slots = np.unique(np.concatenate([vp_row[parent[ce[b0:b1]]] for b0, b1 in part]))
        a0 = int(slots[0]) & ~3
        n4 = (_round4(int(slots[-1]) + 1) - a0) // 4
        blk = np.zeros((n4 * 4, 4), dtype=np.float32)  # [slot][dim]
        for jj, (b0, b1) in enumerate(part):
            e = ce[b0:b1]
            blk[vp_row[parent[e]] - a0, jj] = C[e, 0]
        ab = np.zeros((2, 4), dtype=np.float32)
        for jj, dd in enumerate(dims4):
            ab[0, jj] = alpha0[dd] * fa[dd]
            ab[1, jj] = alpha0[dd] * fb[dd]
        while len(dims4) < 4:
            dims4.append(dims4[0])
        blk_dims.append(dims4)
        blk_run.append((a0, n4, runs.ncoef, 0))
        runs.coef.append(blk.ravel())
        runs.ncoef += blk.size
        blk_ab.append(ab.ravel())
        cost_blk.append(16.0 + 9.0 * n4)
    # general cold groups: runs carry the degree
    cold_tab, cold_ab, cost_cold = [], [], []
    for i, j in general:
        dd = dim[ce[i]]
        r_first = len(runs.tab)
        c = 8.0
        q = i
        while q < j:
            g = deg[ce[q]]
            q2 = q
            while q2 < j and deg[ce[q2]] == g:
                q2 += 1
            grp = ce[q:q2]
            r0, r1 = runs.add(vp_row[parent[grp]], C[grp], degree=int(g))
            c += sum(3 + t[1] / 4.0 * (1 + d_out) for t in runs.tab[r0:r1])
            q = q2
        cold_tab.append((int(dd), r_first, len(runs.tab), int(deg[ce[i:j]].max()) | (int(fam[dd]) << 16)))
        cold_ab.append((fa[dd], fb[dd]))
        cost_cold.append(c)

    allowed_nodes = [i for i in range(nodes.size + 1) if i == nodes.size or level[nodes[i]] <= 1]
    node_seg = _cuts(cost_nodes, allowed_nodes, nseg)
    cold_seg = _cuts(np.asarray(cost_cold), list(range(len(cost_cold) + 1)), nseg)
    block_seg = _cuts(np.asarray(cost_blk), list(range(len(cost_blk) + 1)), nseg)
    as_i32 = lambda v, w: np.asarray(v, dtype=np.int64).reshape(-1, w).astype(np.int32)
    return dict(
        dstride=dstride, row=row, n_hb=n_hb, n_vp=n_vp, n_hot_dims=int(hot_dims.size), n_nodes=int(nodes.size),
        n_cold_groups=len(cold_tab), max_depth=max_depth, node_seg=node_seg, cold_seg=cold_seg,
        n_cold_blocks=len(blk_dims), block_seg=block_seg,
        blk_dims=as_i32(blk_dims, 4) if blk_dims else np.zeros((0, 4), np.int32),
        blk_run=as_i32(blk_run, 4) if blk_run else np.zeros((0, 4), np.int32),
        blk_ab=np.asarray(blk_ab, dtype=np.float32).reshape(-1, 8),
        cold_ab=np.asarray(cold_ab, dtype=np.float32).reshape(-1, 2),
        hot_dim=hot_dims.astype(np.int32), hot_deg=hot_deg.astype(np.int32), hot_soff=hot_soff.astype(np.int32),
        node=as_i32(node_tab, 4), node_c=node_c, cold=as_i32(cold_tab, 4) if cold_tab else np.zeros((0, 4), np.int32),
        run=as_i32(runs.tab, 4) if runs.tab else np.zeros((0, 4), np.int32),
        coef=np.concatenate(runs.coef) if runs.coef else np.zeros(4, np.float32),
        cost=dict(nodes=float(cost_nodes.sum()), cold=float(np.sum(cost_cold)), blocks=float(np.sum(cost_blk)),
                  runs=len(runs.tab), coef_floats=int(runs.ncoef), node_seg=node_seg, cold_seg=cold_seg,
                  block_seg=block_seg),
    )


def build_layout64(tr, C, maxdeg, d, fam, fa, fb, nseg=4):
    """Layout of the FP64 evaluator of the orthogonal form (``csrc/spectral64.cu``):
    the per-point structure of ``build_layout`` with every entry of Lambda as
    exactly one term (row slot, FP64 coefficients) and no padding -- at GB300's
    FP64 rate every term is a multiply-add that counts.  Hot nodes (DFS
    pre-order) carry the terms of their hot leaf children; each cold dimension
    is a group whose runs (one per degree) hold the terms over the prefix
    slots.  ``terms`` is [n_terms, 2] FP64 with the slot's integer bits in
    column 0 and, for one output, the coefficient in column 1; with several
    outputs the coefficients are ``coef`` [n_terms, dstride].  C: FP64
    coefficients [entry] or [entry, d_out]."""
    C = np.asarray(C, dtype=np.float64)
    C = C.reshape(C.shape[0], -1)
    d_out = C.shape[1]
    dstride = 1 if d_out == 1 else _round4(d_out)
    fr = _layout_front(tr, maxdeg, d)
    dim, deg, level, parent = fr["dim"], fr["deg"], fr["level"], fr["parent"]
    n_hb, n_vp, nodes, slot, vp_row = fr["n_hb"], fr["n_vp"], fr["nodes"], fr["slot"], fr["vp_row"]
    leaf_e, starts, ends, cold_e = fr["leaf_e"], fr["starts"], fr["ends"], fr["cold_e"]
    row = (n_hb + n_vp) | 1  # odd: 8-byte row reads of 16 consecutive points fall on distinct banks
    t_slot, t_ent = [], []
    node_tab = np.zeros((nodes.size, 4), dtype=np.int64)
    node_c = np.zeros((nodes.size, dstride))
    cost_nodes = np.zeros(nodes.size)
    for i, e in enumerate(nodes):
        le = leaf_e[starts[i] : ends[i]]
        t0 = len(t_slot)
        t_slot.extend(slot[le].tolist())
        t_ent.extend(le.tolist())
        sl = int(slot[e]) if e != 0 else 0
        node_tab[i] = (sl | (int(level[e]) << 16), int(vp_row[e]) if e != 0 and vp_row[e] >= 0 else -1, t0,
                       len(t_slot))
        if e != 0:  # the root's coefficients are c0
            node_c[i, :d_out] = C[e]
        cost_nodes[i] = 4 + le.size
    ce = cold_e[np.lexsort((vp_row[parent[cold_e]], deg[cold_e], dim[cold_e]))] if cold_e.size else cold_e
    cold_tab, cold_ab, runs, cost_cold = [], [], [], []
    i = 0
    while i < ce.size:
        j = i
        while j < ce.size and dim[ce[j]] == dim[ce[i]]:
            j += 1
        dd = int(dim[ce[i]])
        r_first = len(runs)
        q = i
        while q < j:
            g = int(deg[ce[q]])
            q2 = q
            while q2 < j and deg[ce[q2]] == g:
                q2 += 1
            grp = ce[q:q2]
            t0 = len(t_slot)
            t_slot.extend(vp_row[parent[grp]].tolist())
            t_ent.extend(grp.tolist())
            runs.append((t0, len(t_slot), g, 0))
            q = q2
        gmax = int(deg[ce[i:j]].max())
        unit = int(fa[dd] == 1.0 and fb[dd] == 0.0)
        cold_tab.append((dd, r_first, len(runs), gmax | (int(fam[dd]) << 16) | (unit << 20)))
        cold_ab.append((fa[dd], fb[dd]))
        cost_cold.append(3.0 + (j - i) + 3.0 * gmax)
        i = j
    allowed_nodes = [q for q in range(nodes.size + 1) if q == nodes.size or level[nodes[q]] <= 1]
    T = len(t_slot)
    terms = np.zeros((max(T, 1), 2))
    terms[:T, 0] = np.asarray(t_slot, dtype=np.int64).view(np.float64)
    coef = np.zeros((0, 1))
    if d_out == 1:
        terms[:T, 1] = C[t_ent, 0]
    else:
        coef = np.zeros((max(T, 1), dstride))
        coef[:T, :d_out] = C[t_ent]
    as_i32 = lambda v, w: np.asarray(v, dtype=np.int64).reshape(-1, w).astype(np.int32)
    return dict(
        d_out=d_out, dstride=dstride, row=row, n_hb=n_hb, n_vp=n_vp, n_hot_dims=int(fr["hot_dims"].size),
        n_nodes=int(nodes.size), n_cold_groups=len(cold_tab), max_depth=fr["max_depth"], n_terms=T,
        node_seg=_cuts(cost_nodes, allowed_nodes, nseg),
        cold_seg=_cuts(np.asarray(cost_cold), list(range(len(cost_cold) + 1)), nseg),
        hot_dim=fr["hot_dims"].astype(np.int32), hot_deg=fr["hot_deg"].astype(np.int32),
        hot_soff=fr["hot_soff"].astype(np.int32), node=as_i32(node_tab, 4), node_c=node_c,
        cold=as_i32(cold_tab, 4) if cold_tab else np.zeros((0, 4), np.int32),
        cold_ab=np.asarray(cold_ab, dtype=np.float64).reshape(-1, 2),
        run=as_i32(runs, 4) if runs else np.zeros((0, 4), np.int32), terms=terms, coef=coef,
    )


def evaluate_layout64(lay, x, fam, fa, fb, c0):
    """Host FP64 replay of the FP64 evaluator's sums over a layout (tests):
    [P, d_out]."""
    P = x.shape[0]
    d_out = lay["d_out"]
    R = np.zeros((P, lay["row"]))
    hd, hg, ho = lay["hot_dim"], lay["hot_deg"], lay["hot_soff"]
    for q in range(hd.size):
        R[:, ho[q] : ho[q] + hg[q]] = _phi_table(int(fam[hd[q]]), fa[hd[q]] * x[:, hd[q]] + fb[hd[q]], int(hg[q]))[1:].T
    R[:, lay["n_hb"]] = 1.0
    T = lay["n_terms"]
    slots = lay["terms"][:T, 0].view(np.int64)
    coef = lay["terms"][:T, 1:2] if d_out == 1 else lay["coef"][:T, :d_out]
    acc = np.tile(np.asarray(c0, dtype=float).reshape(1, -1), (P, 1))
    stack = [np.ones(P)] * 9
    for i, nd in enumerate(lay["node"]):
        depth = int(nd[0]) >> 16
        v = np.ones(P) if depth == 0 else (R[:, int(nd[0]) & 0xFFFF] if depth == 1 else stack[depth - 1] * R[:, int(nd[0]) & 0xFFFF])
        stack[depth] = v
        if nd[1] >= 0:
            R[:, nd[1]] = v
        s = lay["node_c"][i, :d_out][None, :] + R[:, slots[nd[2] : nd[3]]] @ coef[nd[2] : nd[3]]
        acc += v[:, None] * s
    for g, cg in enumerate(lay["cold"]):
        dd, r0, r1, w = (int(v) for v in cg)
        z = lay["cold_ab"][g, 0] * x[:, dd] + lay["cold_ab"][g, 1]
        gmax = w & 0xFFFF
        ph = _phi_table((w >> 16) & 0xF, z, gmax)
        for r in range(r0, r1):
            t0, t1, gg, _ = (int(v) for v in lay["run"][r])
            acc += ph[gg][:, None] * (R[:, slots[t0:t1]] @ coef[t0:t1])
    return acc


def evaluate_layout(lay, x, fam, fa, fb, c0):
    """Host FP64 evaluation of a layout: the kernel's arithmetic, for testing the builder."""
    P = x.shape[0]
    d_out = c0.shape[0]
    ds = lay["dstride"]
    out = np.tile(np.asarray(c0, dtype=float), (P, 1))

    def phis(dim, g):
        z = fa[dim] * x[:, dim] + fb[dim]
        vals, pm1, pc = [], np.zeros(P), np.ones(P)
        for m in range(g):
            if fam[dim] == 0:
                al, be = (2 * m + 1) / (m + 1), m / (m + 1)
            else:
                al, be = np.sqrt(2 / (m + 1)), np.sqrt(m / (m + 1))
            pm1, pc = pc, al * z * pc - be * pm1
            vals.append(pc)
        return vals

    R = np.zeros((P, lay["row"]))
    for h in range(lay["n_hot_dims"]):
        vals = phis(int(lay["hot_dim"][h]), int(lay["hot_deg"][h]))
        for m, v in enumerate(vals):
            R[:, lay["hot_soff"][h] + m] = v
    R[:, lay["n_hb"]] = 1.0

    def dot(r0, r1):
        s = np.zeros((P, d_out))
        for r in range(r0, r1):
            st, ln, co, _ = lay["run"][r]
            blk = lay["coef"][co : co + ln * ds].reshape(ln, ds)[:, :d_out].astype(float)
            s += R[:, st : st + ln] @ blk
        return s

    stack = [np.ones(P)] * 9
    for i in range(lay["n_nodes"]):
        w, vp, r0, r1 = lay["node"][i]
        depth, sl = int(w) >> 16, int(w) & 0xFFFF
        if depth == 0:
            v = np.ones(P)
        else:
            v = stack[depth - 1] * R[:, sl]
            stack[depth] = v
        if vp >= 0:
            R[:, vp] = v
        out += v[:, None] * (lay["node_c"][i, :d_out][None, :] + dot(r0, r1))
    for bi in range(lay["n_cold_blocks"]):
        dims4 = lay["blk_dims"][bi]
        a0, n4, co, _ = lay["blk_run"][bi]
        blk = lay["coef"][co : co + 16 * n4].reshape(4 * n4, 4).astype(float)
        u = R[:, a0 : a0 + 4 * n4] @ blk  # (P, 4)
        ab = lay["blk_ab"][bi].reshape(2, 4)
        phi = np.stack([ab[0, j] * x[:, dims4[j]] + ab[1, j] for j in range(4)], axis=1)
        out[:, 0] += np.sum(phi * u, axis=1)
    for gi in range(lay["n_cold_groups"]):
        dd, r0, r1, gmax = lay["cold"][gi]
        vals = phis(int(dd), int(gmax) & 0xFF)
        for r in range(r0, r1):
            out += vals[lay["run"][r][3] - 1][:, None] * dot(r, r + 1)
    return out

