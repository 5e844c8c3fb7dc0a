"""Host logic of the tensor-core blocked evaluator's tables (no GPU needed).

The library's builder (``smx_layout_build``, kind ``blocked_tc``) stores the
coefficients as three bf16 parts in the swizzled shared-memory image of the
MMA's B operand.  The test decodes that image, replays the evaluator's sum in
FP64 (basis values of the table slots, prefix products of the rows, the
table and linear columns) and compares it with the direct sum over the index
set; it also checks the staircase (no coefficient outside a chunk's K
extent), the stage order and the x-box masks.
"""
import numpy as np
import pytest

from smolyax_gb300 import _capi as capi
from test_layout_cpu import direct, python_tree

I32 = ("tc_td", "tc_row", "tc_chunk", "tc_b", "tc_box")
F32 = ("tc_tdab",)
SCAL = ("tc_n_td", "tc_n_phi", "tc_n_phi_pad", "tc_n_rows", "tc_max_depth", "tc_n_agen", "tc_kt_table", "tc_n_chunks",
        "tc_n_boxes", "tc_lin0", "tc_stages", "tc_smem", "c0")


def _bf16(u16):
    return (u16.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def decode(lay):
    """Coefficient matrices (table [rows x n_phi_pad], linear [rows x n_cols]) from the stage image."""
    img = lay["tc_b"].view(np.uint16)
    n_rows = int(lay["tc_n_rows"])
    chunks = lay["tc_chunk"].reshape(-1, 4)
    n_cols = int(lay["tc_n_boxes"]) * 8
    K_all = 16 * max(int(lay["tc_n_agen"]), 1)
    Bt = np.zeros((K_all, int(lay["tc_n_phi_pad"])))
    Bl = np.zeros((K_all, n_cols))
    stage_ks = []
    for c in chunks:
        N, table, nk, off = int(c[0]) & 0xFFFF, int(c[0]) >> 16, int(c[1]), int(c[2]) * 8
        order = list(range(nk - 1, -1, -1))
        stage_ks.append(order)
        for i, kk in enumerate(order):
            st = img[off + i * 3 * N * 16: off + (i + 1) * 3 * N * 16].reshape(3, N, 16)
            nn = np.arange(N)[:, None]
            k = np.arange(16)[None, :]
            pos = (((k >> 3) ^ ((nn >> 2) & 1)) << 3) + (k & 7)
            vals = sum(_bf16(st[sp][nn, pos]) for sp in range(3))  # [N][16]: column nn, row kk*16 + k
            if table:
                Bt[kk * 16: kk * 16 + 16, int(c[3]): int(c[3]) + N] = vals.T
            else:
                col0 = int(c[3]) * 8
                Bl[kk * 16: kk * 16 + 16, col0: col0 + N] = vals.T
    assert not Bt[n_rows:].any() and not Bl[n_rows:].any()
    return Bt[:n_rows], Bl[:n_rows], stage_ks


def replay(lay, x, fam):
    P, d = x.shape
    n_phi_pad = int(lay["tc_n_phi_pad"])
    phi = np.zeros((n_phi_pad, P))
    phi[0] = 1.0
    td = lay["tc_td"].reshape(-1, 4)
    ab = lay["tc_tdab"].reshape(-1, 2).astype(np.float64)
    for (j, g, so, fm), (a, b) in zip(td, ab):
        z = a * x[:, j] + b
        pm1, pc = np.zeros(P), np.ones(P)
        for m in range(g):
            al, be = ((2 * m + 1) / (m + 1), m / (m + 1)) if fm == 0 else (np.sqrt(2 / (m + 1)), np.sqrt(m / (m + 1)))
            pm1, pc = pc, al * z * pc - be * pm1
            phi[so + m] = pc
    rows = lay["tc_row"].reshape(-1, 4).view(np.uint32)
    slots = np.stack([(rows[:, q // 2] >> (16 * (q % 2))) & 0xFFFF for q in range(8)], axis=1)
    V = np.prod(phi[slots], axis=1)  # [rows][P]
    Bt, Bl, _ = decode(lay)
    lin0 = int(lay["tc_lin0"])
    n_cols = Bl.shape[1]
    xl = np.zeros((P, n_cols))
    w = min(n_cols, d - lin0)
    xl[:, :w] = x[:, lin0: lin0 + w]
    mask = np.zeros(n_cols, dtype=bool)
    for b, m in enumerate(lay["tc_box"]):
        for i in range(8):
            mask[8 * b + i] = bool((int(m) >> i) & 1)
    xl[:, mask] = 0.0
    y = float(lay["c0"]) + np.einsum("rp,rs,sp->p", V, Bt, phi) + np.einsum("rp,rc,pc->p", V, Bl, xl)
    return y


def _build(d, t, fam_id, seed, fb_scale=0.2):
    k = list(np.log((2 + np.arange(d)) / np.log(2)))
    tr = python_tree(k, t)
    n = tr["parent"].shape[0]
    rng = np.random.default_rng(seed)
    C = rng.normal(size=(n, 1)).astype(np.float32)
    maxdeg = np.zeros(d, dtype=np.int64)
    np.maximum.at(maxdeg, tr["dim"][1:], tr["deg"][1:])
    fam = np.full(d, fam_id, np.int32)
    fa, fb = rng.uniform(0.5, 1.5, d), rng.uniform(-fb_scale, fb_scale, d)
    lay = capi.host_layout("blocked_tc", tr, C, 1, maxdeg, fam, fa, fb, i32=I32, f32=F32, scalars=SCAL)
    return tr, C, maxdeg, fam, fa, fb, lay


@pytest.mark.parametrize("d,t,fam_id", [(3, 4.5, 0), (12, 6.0, 0), (40, 5.5, 0), (60, 5.8, 1), (200, 6.5, 0),
                                        (300, 7.0, 1), (1000, 8.22452, 0)])
def test_tables_match_direct_sum(d, t, fam_id):
    tr, C, maxdeg, fam, fa, fb, lay = _build(d, t, fam_id, seed=d)
    assert lay is not None
    rng = np.random.default_rng(d + 1)
    x = rng.uniform(-1, 1, (48, d))
    ref = direct(tr, C.astype(np.float64), x, fam, fa, fb)[:, 0]
    got = replay(lay, x, fam)
    # table dimensions use the FP32 affine maps, the folded linear columns FP32 coefficients
    assert np.abs(got - ref).max() <= 1e-6 * max(1.0, np.abs(ref).max())


def test_headline_structure():
    """d = 1000, |Lambda| = 9999: 959 linear dimensions in 15 chunks of 64
    whose K steps follow the staircase, and 41 table dimensions (100 slots:
    two table chunks over every node, 13 K steps) placed after the 5th and
    10th linear chunk; A fits tensor memory with three accumulators."""
    tr, C, maxdeg, fam, fa, fb, lay = _build(1000, 8.22452, 0, seed=0)
    assert int(lay["tc_n_td"]) == 41 and int(lay["tc_n_rows"]) == 208 and int(lay["tc_n_phi"]) == 100
    chunks = lay["tc_chunk"].reshape(-1, 4)
    table = chunks[:, 0] >> 16
    assert list(np.nonzero(table)[0]) == [5, 11] and len(chunks) == 17  # after 5 and 10 linear chunks
    assert list(chunks[table == 1, 1]) == [13, 13] and list(chunks[table == 1, 3]) == [0, 64]
    assert int(lay["tc_n_agen"]) == 13 and 3 * 64 + 24 * 13 <= 512
    assert int(lay["tc_lin0"]) % 8 == 0 and int(lay["tc_n_boxes"]) * 8 >= 1000 - int(lay["tc_lin0"])
    assert int(lay["tc_smem"]) <= 225 * 1024
    Bt, Bl, stage_ks = decode(lay)
    # staircase: every linear chunk's coefficients lie within its K steps, which shrink along the columns
    nks = []
    for c, ks, t in zip(chunks, stage_ks, table):
        if t:
            continue
        col0, N, nk = int(c[3]) * 8, int(c[0]) & 0xFFFF, int(c[1])
        assert not Bl[16 * nk:, col0: col0 + N].any()
        assert ks == list(range(nk - 1, -1, -1))
        nks.append(nk)
    assert nks == sorted(nks, reverse=True) and nks[-1] == 1
    assert int(lay["tc_stages"]) == sum(len(k) for k in stage_ks)
    assert not lay["tc_box"].any()  # 1000 - 40 = 960 linear columns: no unit past d


def test_fold_of_the_affine_constant():
    """With fb = 0 the table chunk's column 0 (the constant slot) holds no folded terms."""
    tr, C, maxdeg, fam, fa, fb, lay = _build(200, 6.5, 0, seed=5, fb_scale=0.0)
    Bt, Bl, _ = decode(lay)
    assert not Bt[:, 0].any()
    x = np.random.default_rng(2).uniform(-1, 1, (16, 200))
    ref = direct(tr, C.astype(np.float64), x, fam, fa, fb)[:, 0]
    assert np.abs(replay(lay, x, fam) - ref).max() <= 1e-6 * max(1.0, np.abs(ref).max())

