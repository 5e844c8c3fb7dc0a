"""Host logic of the FP32 evaluator's layout (no GPU needed).

A small index-set tree is built in Python with the same entry layout as the
device enumeration (root first, children by dimension then degree, parent
ids, remaining budget, pre-order rank); random coefficients are laid out by
``build_layout`` and the run-based evaluation (host FP64 replay of the
kernel's arithmetic) is compared with the direct sum over the index set.
"""
import numpy as np
import pytest

from smolyax_gb300.spectral import build_layout, evaluate_layout


def python_tree(k, t):
    d = len(k)
    ent = [dict(rem=t, start=0, parent=-1, dim=-1, deg=0, level=0)]
    cur = [0]
    while cur:
        nxt = []
        for e in cur:
            E = ent[e]
            i = E["start"]
            if i < d:
                while True:
                    j = 1
                    while j * k[i] < E["rem"]:
                        nxt.append(dict(rem=E["rem"] - j * k[i], start=i + 1, parent=e, dim=i, deg=j,
                                        level=E["level"] + 1))
                        j += 1
                    if i + 1 < d and k[i + 1] < E["rem"]:
                        i += 1
                    else:
                        break
        base = len(ent)
        ent.extend(nxt)
        cur = list(range(base, len(ent)))
    n = len(ent)
    children = [[] for _ in range(n)]
    for e in range(1, n):
        children[ent[e]["parent"]].append(e)
    rank = np.zeros(n, dtype=np.int64)
    order = []

    def visit(e):
        order.append(e)
        for c in children[e]:
            visit(c)

    visit(0)
    rank[np.array(order)] = np.arange(n)
    arr = lambda key: np.array([E[key] for E in ent])
    return dict(parent=arr("parent"), dim=arr("dim"), deg=arr("deg"), level=arr("level"), rank=rank,
                rem=arr("rem").astype(float))


def direct(tr, C, x, fam, fa, fb):
    n = tr["parent"].shape[0]
    P = x.shape[0]
    vals = np.ones((n, P))
    for e in range(1, n):
        dd, g = tr["dim"][e], tr["deg"][e]
        z = fa[dd] * x[:, dd] + fb[dd]
        pm1, pc = np.zeros(P), np.ones(P)
        for m in range(g):
            al, be = ((2 * m + 1) / (m + 1), m / (m + 1)) if fam[dd] == 0 else (np.sqrt(2 / (m + 1)), np.sqrt(m / (m + 1)))
            pm1, pc = pc, al * z * pc - be * pm1
        vals[e] = vals[tr["parent"][e]] * pc
    return vals.T @ C


@pytest.mark.parametrize("d,t,d_out,fam_id", [(3, 4.5, 1, 0), (6, 5.0, 2, 1), (12, 6.0, 1, 0), (40, 5.5, 3, 0),
                                               (60, 5.8, 1, 1), (200, 6.5, 1, 0)])
def test_layout_matches_direct_sum(d, t, d_out, fam_id):
    k = list(np.log((2 + np.arange(d)) / np.log(2)))
    tr = python_tree(k, t)
    n = tr["parent"].shape[0]
    rng = np.random.default_rng(d)
    C = rng.normal(size=(n, d_out)).astype(np.float32)
    maxdeg = np.zeros(d, dtype=np.int64)
    for e in range(1, n):
        maxdeg[tr["dim"][e]] = max(maxdeg[tr["dim"][e]], tr["deg"][e])
    fam = np.full(d, fam_id)
    fa, fb = np.full(d, 0.9), np.full(d, 0.05)
    lay = build_layout(tr, C, maxdeg, d, d_out, fam, fa, fb)
    x = rng.uniform(-1, 1, (7, d))
    ref = direct(tr, C.astype(float), x, fam, fa, fb)
    got = evaluate_layout(lay, x, fam, fa, fb, C[0].astype(float))
    # blocks hold their affine maps in FP32 (as the kernel reads them): 1e-6
    scale = np.max(np.abs(ref))
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6 * scale)
    # structural invariants the kernel relies on
    assert lay["row"] % 4 == 0 and lay["row"] >= lay["n_hb"] + lay["n_vp"]
    assert all(r[0] % 4 == 0 and r[1] % 4 == 0 and r[0] + r[1] <= lay["row"] for r in lay["run"])
    assert lay["node_seg"][0] == 0 and lay["node_seg"][-1] == lay["n_nodes"]
    assert lay["cold_seg"][0] == 0 and lay["cold_seg"][-1] == lay["n_cold_groups"]
    assert np.all(np.diff(lay["node_seg"]) >= 0) and np.all(np.diff(lay["cold_seg"]) >= 0)
    assert lay["max_depth"] <= 8
    assert lay["block_seg"][-1] == lay["n_cold_blocks"] and (d_out == 1 or lay["n_cold_blocks"] == 0)


@pytest.mark.parametrize("d,t,fam_id,unit,d_out", [(1, 3.0, 0, False, 1), (3, 4.5, 0, True, 1), (6, 5.0, 1, False, 3),
                                                   (12, 6.0, 0, True, 1), (60, 5.8, 1, False, 1), (40, 5.5, 0, False, 6),
                                                   (200, 6.5, 0, True, 1), (1000, 8.22452, 0, True, 1)])
def test_fp64_layout_matches_direct_sum(d, t, fam_id, unit, d_out):
    """The FP64 evaluator's layout (``build_layout64``): every entry of the
    index set is exactly one term (no padding), the sums replayed in FP64 equal
    the direct sum over the tree to rounding, and the row, term and segment
    invariants the kernel relies on hold."""
    from smolyax_gb300.spectral import build_layout64, evaluate_layout64

    k = list(np.log((2 + np.arange(d)) / np.log(2)))
    tr = python_tree(k, t)
    n = tr["parent"].shape[0]
    rng = np.random.default_rng(d + 7)
    C = rng.normal(size=(n, d_out))
    maxdeg = np.zeros(d, dtype=np.int64)
    for e in range(1, n):
        maxdeg[tr["dim"][e]] = max(maxdeg[tr["dim"][e]], tr["deg"][e])
    fam = np.full(d, fam_id)
    fa, fb = (np.ones(d), np.zeros(d)) if unit else (np.full(d, 0.9), np.full(d, 0.05))
    lay = build_layout64(tr, C, maxdeg, d, fam, fa, fb)
    x = rng.uniform(-1, 1, (5, d))
    ref = direct(tr, C, x, fam, fa, fb)
    got = evaluate_layout64(lay, x, fam, fa, fb, C[0])
    assert lay["d_out"] == d_out and lay["dstride"] == (1 if d_out == 1 else (d_out + 3) // 4 * 4)
    if d_out > 1:
        assert lay["coef"].shape == (lay["n_terms"], lay["dstride"]) and np.all(lay["coef"][:, d_out:] == 0)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.max(np.abs(ref)))
    # one term per entry: all entries but the root and the hot nodes
    assert lay["n_terms"] == n - lay["n_nodes"]
    slots = lay["terms"][: lay["n_terms"], 0].view(np.int64)
    assert slots.min(initial=0) >= 0 and slots.max(initial=0) < lay["n_hb"] + lay["n_vp"] <= lay["row"]
    assert lay["row"] % 2 == 1
    node = lay["node"]
    assert np.all(node[:, 2] <= node[:, 3]) and np.all(slots[np.concatenate(
        [np.arange(a, b) for a, b in node[:, 2:4]] + [np.zeros(0, np.int64)]).astype(np.int64)] < lay["n_hb"])
    assert lay["node_seg"][0] == 0 and lay["node_seg"][-1] == lay["n_nodes"]
    assert lay["cold_seg"][0] == 0 and lay["cold_seg"][-1] == lay["n_cold_groups"]
    assert np.all(np.diff(lay["node_seg"]) >= 0) and np.all(np.diff(lay["cold_seg"]) >= 0)
    assert all((int(c[3]) >> 20) & 1 == int(unit) and (int(c[3]) >> 16) & 0xF == fam_id for c in lay["cold"])
