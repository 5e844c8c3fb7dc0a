"""Host logic of the blocked FP32 evaluator's tables (no GPU needed).

The tables built by ``build_blocked`` are replayed on the host in FP64 (the
kernel's sums: hot gather per node, staircase blocks of the cold groups) and
compared with the direct sum over the index set; work lists must cover every
item once.
"""
import numpy as np
import pytest

from smolyax_gb300.blocked import N_WARPS, build_blocked, replay_blocked
from test_layout_cpu import direct, python_tree


@pytest.mark.parametrize("d,t,fam_id", [(1, 3.0, 0), (3, 4.5, 0), (6, 5.0, 1), (12, 6.0, 0), (40, 5.5, 0),
                                        (60, 5.8, 1), (200, 6.5, 0), (1000, 8.22452, 0)])
def test_blocked_tables_match_direct_sum(d, t, fam_id):
    k = list(np.log((2 + np.arange(d)) / np.log(2)))
    tr = python_tree(k, t)
    n = tr["parent"].shape[0]
    rng = np.random.default_rng(d)
    C = rng.normal(size=(n, 1)).astype(np.float32)
    maxdeg = np.zeros(d, dtype=np.int64)
    np.maximum.at(maxdeg, tr["dim"][1:], tr["deg"][1:])
    fam = np.full(d, fam_id, np.int32)
    fa, fb = rng.uniform(0.5, 1.5, d), rng.uniform(-0.2, 0.2, d)
    lay = build_blocked(tr, C[:, 0], maxdeg, d, fam, fa, fb)
    assert lay is not None
    x = rng.uniform(-1, 1, (64, d))
    ref = direct(tr, C.astype(np.float64), x, fam, lay["fa"].astype(np.float64), lay["fb"].astype(np.float64))[:, 0]
    got = replay_blocked(lay, x, fam)
    # fast groups hold alpha_0 * a in FP32: Hermite rounding differs from the direct sum's
    tol = 1e-14 if fam_id == 0 else 1e-7
    assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max())
    # every hot node with entries and every cold group appears in exactly one warp's list
    items = lay["items"]
    assert lay["warp_off"].shape[0] == N_WARPS + 1 and lay["warp_off"][-1] == items.size
    cold = np.sort(items[items >= (1 << 30)] - (1 << 30))
    assert np.array_equal(cold, np.arange(lay["n_groups"]))
    hot = np.sort(items[items < (1 << 30)])
    node = lay["node"].reshape(-1, 12)
    assert np.array_equal(hot, np.nonzero(node[:, 1] > 0)[0])
    assert lay["smem"] == (lay["n_hs"] + lay["k_c"]) * 512 + 2 * N_WARPS * 512
    # the kernel's 16- and 32-byte x loads of a "fast" group start at its first
    # dimension: it must be a multiple of 4, the dimensions consecutive, degree 1
    grp = lay["grp"].reshape(-1, 12)
    for g in grp[grp[:, 2] != 0]:
        dims, degs = g[4:8], g[8:12]
        assert dims[0] % 4 == 0 and np.array_equal(dims, dims[0] + np.arange(4)) and np.all(degs == 1)


def test_blocked_balance_at_high_dimension():
    d, t = 1000, 8.22452
    k = list(np.log((2 + np.arange(d)) / np.log(2)))
    tr = python_tree(k, t)
    n = tr["parent"].shape[0]
    maxdeg = np.zeros(d, dtype=np.int64)
    np.maximum.at(maxdeg, tr["dim"][1:], tr["deg"][1:])
    lay = build_blocked(tr, np.ones(n, np.float32), maxdeg, d, np.zeros(d, np.int32), np.ones(d), np.zeros(d))
    assert lay["n_hs"] == 97 and lay["k_c"] == 71
    assert lay["load_max"] / lay["load_mean"] < 1.02
    grp = lay["grp"].reshape(-1, 12)
    assert grp[:, 2].sum() >= grp.shape[0] - 2  # nearly every cold group reads x as 2 x 16 bytes per point
