"""Layout of the blocked FP32 evaluator (``csrc/blocked.cu``), one output.

The orthogonal form I(x) = c_0 + sum_{e != root} c_e V_{parent(e)}(x) phi_{slot(e)}(x)
is split by the kind of the last factor of every entry e:

* hot entries (last dimension hot, i.e. a dimension that has children in the
  index set; with k sorted ascending the hot dimensions are 0..H-1) are summed
  per parent node: y += V_a * sum_{(a, s)} c * Phi[s], with Phi[s] the
  per-point basis value of hot slot s (a table in shared memory) and V_a the
  product of the basis values along the path of node a;
* cold entries (last dimension cold) extend a prefix a whose value V_a is one
  of K_c "prefix rows".  Sorted by remaining budget (descending), the prefixes
  admissible for a cold slot (j, g) are exactly the first L_(j,g) ones (a
  prefix admits (j, g) iff g * k_j < rem(a)), so the coefficients of a group of
  4 cold slots form a staircase block W[K][4], K = the largest L in the group:
  T[p][s] = sum_k Vc[k][p] W[k][s], then y += sum_s T[p][s] phi_s(x_p).

Work items (hot nodes, cold groups) are assigned to the 16 warps of a block
by a greedy balance of an instruction-count estimate; every warp covers all
128 points of a tile (lane l: points l, l+32, l+64, l+96).
"""
from __future__ import annotations

import numpy as np

N_WARPS = 16
TILE = 128
MAX_PATH = 8
SMEM_LIMIT = 220 * 1024


def _alpha0(fam):
    """phi_1 = alpha_0 * z (Legendre 1, normalised Hermite sqrt(2))."""
    return 1.0 if fam == 0 else np.sqrt(2.0)


def smem_bytes(n_hs, k_c):
    return (int(n_hs) + int(k_c)) * TILE * 4 + 2 * N_WARPS * TILE * 4


def build_blocked(tr, C, maxdeg, d, fam, fa, fb):
    """Layout from the index-set tree (host arrays parent, dim, deg, rem) and the
    FP32 coefficients C[entry] (one output).  Returns None when the plan is
    outside what the kernel handles (path deeper than 8, shared memory)."""
    parent, dim, deg, rem = (np.asarray(tr[key]) for key in ("parent", "dim", "deg", "rem"))
    C = np.asarray(C, dtype=np.float32).reshape(-1)
    n = parent.shape[0]
    maxdeg = np.asarray(maxdeg, dtype=np.int64)
    e = np.arange(1, n)

    hot = np.zeros(d, dtype=bool)
    inner = e[parent[e] > 0]
    hot[dim[parent[inner]]] = True
    hot_dims = np.nonzero(hot)[0]
    hot_deg = maxdeg[hot_dims]
    hot_soff = np.concatenate([[0], np.cumsum(hot_deg)[:-1]]).astype(np.int64) if hot_dims.size else \
        np.zeros(0, np.int64)
    n_hs = int(hot_deg.sum())
    hidx = np.full(d, -1, dtype=np.int64)
    hidx[hot_dims] = np.arange(hot_dims.size)
    is_hot_e = hot[dim[e]]
    hot_e, cold_e = e[is_hot_e], e[~is_hot_e]

    # hot slot of every hot entry; path of slots from the root
    hslot = np.full(n, -1, dtype=np.int64)
    hslot[hot_e] = hot_soff[hidx[dim[hot_e]]] + deg[hot_e] - 1
    has_kid = np.zeros(n, dtype=bool)
    has_kid[parent[e]] = True
    nodes = np.nonzero(has_kid)[0]
    if nodes.size == 0 or nodes[0] != 0:
        nodes = np.concatenate([[0], nodes[nodes != 0]])
    depth = np.zeros(n, dtype=np.int64)
    paths = {0: []}
    for a in nodes[1:]:
        p = []
        v = a
        while v != 0:
            p.append(int(hslot[v]))
            v = parent[v]
        if len(p) > MAX_PATH or min(p) < 0:
            return None
        paths[int(a)] = p[::-1]
        depth[a] = len(p)
    nidx = np.full(n, -1, dtype=np.int64)
    nidx[nodes] = np.arange(nodes.size)

    # hot entries grouped by parent node, two per 16 bytes
    order = hot_e[np.lexsort((hslot[hot_e], nidx[parent[hot_e]]))]
    node_tab = np.zeros((nodes.size, 12), dtype=np.int32)
    ent = []
    cnt = np.bincount(nidx[parent[order]], minlength=nodes.size) if order.size else np.zeros(nodes.size, np.int64)
    pos = 0
    for i, a in enumerate(nodes):
        sel = order[pos : pos + cnt[i]]
        pos += cnt[i]
        node_tab[i, 0] = len(ent)
        for v in sel:
            ent.append((int(hslot[v]) * TILE, float(C[v])))
        if len(sel) % 2:
            ent.append((0, 0.0))
        node_tab[i, 1] = len(ent) - node_tab[i, 0]
        node_tab[i, 2] = depth[a]
        pth = paths[int(a)]
        node_tab[i, 4 : 4 + len(pth)] = np.asarray(pth, dtype=np.int32) * TILE
    ent_off = np.array([o for o, _ in ent], dtype=np.int32)
    ent_c = np.array([c for _, c in ent], dtype=np.float32)
    hot_ent = np.empty(2 * len(ent), dtype=np.int32)
    hot_ent[0::2] = ent_off
    hot_ent[1::2] = ent_c.view(np.int32)

    # prefix rows of the cold entries, by remaining budget (descending)
    pref = np.unique(parent[cold_e]) if cold_e.size else np.zeros(0, np.int64)
    if pref.size:
        pref = pref[np.lexsort((pref, -rem[pref]))]
    k_c = int(pref.size)
    kc = np.full(n, -1, dtype=np.int64)
    kc[pref] = np.arange(k_c)
    vc_tab = node_tab[nidx[pref]].copy() if k_c else np.zeros((0, 12), np.int32)
    if smem_bytes(n_hs, k_c) > SMEM_LIMIT:
        return None

    # cold slots: staircase check, then groups over windows of 4 dimensions
    coef_of = {}
    L = {}
    for v in cold_e:
        s = (int(dim[v]), int(deg[v]))
        coef_of[(int(kc[parent[v]]), s)] = float(C[v])
        L[s] = L.get(s, 0) + 1
    for (k, s) in coef_of:
        if k >= L[s]:
            return None  # admissible prefixes are not a leading range
    slots = sorted(L)
    groups = []
    i = 0
    while i < len(slots):
        w = slots[i][0] // 4
        j = i
        while j < len(slots) and slots[j][0] // 4 == w:
            j += 1
        win = slots[i:j]
        fast = len(win) == 4 and all(s[1] == 1 for s in win) and [s[0] for s in win] == list(range(4 * w, 4 * w + 4))
        for q in range(0, len(win), 4):
            groups.append((win[q : q + 4], fast))
        i = j
    grp = np.zeros((len(groups), 12), dtype=np.int32)
    grp_ab = np.zeros((len(groups), 8), dtype=np.float32)
    W = []
    for g, (sl, fast) in enumerate(groups):
        K = max(L[s] for s in sl)
        grp[g, 0] = K
        grp[g, 1] = len(W)
        grp[g, 2] = 1 if fast else 0
        grp[g, 3] = len(sl)
        for q in range(4):
            if q < len(sl):
                j_, g_ = sl[q]
                grp[g, 4 + q] = j_
                grp[g, 8 + q] = g_
                if fast:
                    a0 = _alpha0(int(fam[j_]))
                    grp_ab[g, q], grp_ab[g, 4 + q] = a0 * fa[j_], a0 * fb[j_]
                else:
                    grp_ab[g, q], grp_ab[g, 4 + q] = fa[j_], fb[j_]
            else:
                grp[g, 4 + q] = sl[0][0]
                grp[g, 8 + q] = 0  # unused slot
        if fast and np.all(grp_ab[g, :4] == np.float32(1.0)) and np.all(grp_ab[g, 4:] == np.float32(0.0)):
            grp[g, 2] = 2  # unit maps: phi_1 = x
        for k in range(K):
            for q in range(4):
                W.append(coef_of.get((k, sl[q]), 0.0) if q < len(sl) else 0.0)
    W = np.asarray(W, dtype=np.float32)

    # items and their balance over the warps
    hot_items = [i for i in range(nodes.size) if node_tab[i, 1] > 0]
    cost_hot = {i: 12 + 6.5 * node_tab[i, 1] + 3 * node_tab[i, 2] for i in hot_items}
    load = np.zeros(N_WARPS)
    lists = [[] for _ in range(N_WARPS)]
    for i in sorted(hot_items, key=lambda i: -cost_hot[i]):
        w = int(np.argmin(load))
        lists[w].append(i)
        load[w] += cost_hot[i]
    for g in range(len(groups)):
        K = grp[g, 0]
        c = 24 + 18 * K + (40 if grp[g, 2] else 100 + 20 * int(grp[g, 8:12].sum()))
        w = int(np.argmin(load))
        lists[w].append((1 << 30) | g)
        load[w] += c
    warp_off = np.zeros(N_WARPS + 1, dtype=np.int32)
    warp_off[1:] = np.cumsum([len(li) for li in lists])
    items = np.asarray([it for li in lists for it in li], dtype=np.int32)

    return dict(
        d_in=d, n_hs=n_hs, k_c=k_c, n_hot_dims=int(hot_dims.size), n_nodes=int(nodes.size),
        n_groups=len(groups), n_items=int(items.size), c0=float(C[0]),
        hot_dim=hot_dims.astype(np.int32), hot_deg=hot_deg.astype(np.int32), hot_soff=hot_soff.astype(np.int32),
        node=node_tab.reshape(-1), vc=vc_tab.reshape(-1), hot_ent=hot_ent, grp=grp.reshape(-1),
        grp_ab=grp_ab.reshape(-1), W=W, warp_off=warp_off, items=items,
        smem=smem_bytes(n_hs, k_c), load_max=float(load.max()), load_mean=float(load.mean()),
        fa=np.asarray(fa, dtype=np.float32), fb=np.asarray(fb, dtype=np.float32),
    )


def _phi(fam, z, g):
    pm1, pc = np.zeros_like(z), np.ones_like(z)
    for m in range(g):
        a, b = ((2 * m + 1) / (m + 1), m / (m + 1)) if fam == 0 else (np.sqrt(2.0 / (m + 1)), np.sqrt(m / (m + 1)))
        pm1, pc = pc, a * z * pc - b * pm1
    return pc


def replay_blocked(lay, x, fam):
    """FP64 host replay of the kernel's sums over the layout (for tests)."""
    x = np.asarray(x, dtype=np.float64)
    P = x.shape[0]
    PH = np.zeros((max(lay["n_hs"], 1), P))
    for h in range(lay["n_hot_dims"]):
        dd, gmax, so = lay["hot_dim"][h], lay["hot_deg"][h], lay["hot_soff"][h]
        z = np.float64(lay["fa"][dd]) * x[:, dd] + np.float64(lay["fb"][dd])
        for g in range(1, gmax + 1):
            PH[so + g - 1] = _phi(int(fam[dd]), z, g)
    node = lay["node"].reshape(-1, 12)
    y = np.full(P, lay["c0"], dtype=np.float64)

    def path_val(row):
        v = np.ones(P)
        for q in range(row[2]):
            v = v * PH[row[4 + q] // TILE]
        return v

    ent = lay["hot_ent"].reshape(-1, 2)
    for i in range(node.shape[0]):
        o, c = node[i, 0], node[i, 1]
        if c == 0:
            continue
        acc = np.zeros(P)
        for q in range(o, o + c):
            acc += np.float64(ent[q, 1:2].view(np.float32)[0]) * PH[ent[q, 0] // TILE]
        y += path_val(node[i]) * acc
    vc = lay["vc"].reshape(-1, 12)
    VC = np.array([path_val(vc[k]) for k in range(vc.shape[0])]) if vc.shape[0] else np.zeros((0, P))
    grp = lay["grp"].reshape(-1, 12)
    ab = lay["grp_ab"].reshape(-1, 8)
    for g in range(grp.shape[0]):
        K, wo, fast, ns = grp[g, :4]
        Wg = lay["W"][wo : wo + 4 * K].reshape(K, 4).astype(np.float64)
        Tm = VC[:K].T @ Wg  # [P][4]
        for q in range(ns):
            dd, gg = grp[g, 4 + q], grp[g, 8 + q]
            if fast:
                phi = ab[g, q] * x[:, dd] + ab[g, 4 + q]
            else:
                phi = _phi(int(fam[dd]), ab[g, q] * x[:, dd] + ab[g, 4 + q], gg)
            y += Tm[:, q] * phi
    return y
