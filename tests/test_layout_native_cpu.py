"""The library's host-side layout builders (``smx_layout_build``, used by the
C-ABI FP32 plan) produce the same tables as the package's Python builders
(blocked evaluator, per-point evaluator, tensor-core tape), bit for bit."""
import numpy as np
import pytest

from smolyax_gb300 import _capi
from smolyax_gb300.blocked import build_blocked
from smolyax_gb300.spectral import build_layout, build_tape
from test_layout_cpu import python_tree


def _case(d, t, d_out, fam_id, seed):
    k = list(np.log((2 + np.arange(d)) / np.log(2)))
    tr = python_tree(k, t)
    n = tr["parent"].shape[0]
    rng = np.random.default_rng(seed)
    C = rng.normal(size=(n, d_out)).astype(np.float32)
    maxdeg = np.zeros(d, dtype=np.int64)
    np.maximum.at(maxdeg, tr["dim"][1:], tr["deg"][1:])
    fam = np.full(d, fam_id, np.int32)
    fam[::3] = 1 - fam_id  # mixed families
    fa, fb = rng.uniform(0.5, 1.5, d), rng.uniform(-0.2, 0.2, d)
    return tr, C, maxdeg, fam, fa, fb


BLOCKED_I32 = ("hot_dim", "hot_deg", "hot_soff", "node", "vc", "hot_ent", "grp", "warp_off", "items")
BLOCKED_F32 = ("grp_ab", "W")
BLOCKED_SCALARS = ("n_hs", "k_c", "n_hot_dims", "n_nodes", "n_groups", "n_items", "c0")


@pytest.mark.parametrize("d,t,fam_id", [(1, 3.0, 0), (6, 5.0, 1), (12, 6.0, 0), (40, 5.5, 0), (60, 5.8, 1),
                                        (200, 6.5, 0), (1000, 8.22452, 0)])
def test_blocked_tables_equal(d, t, fam_id):
    tr, C, maxdeg, fam, fa, fb = _case(d, t, 1, fam_id, d)
    py = build_blocked(tr, C[:, 0], maxdeg, d, fam, fa, fb)
    nat = _capi.host_layout("blocked", tr, C, 1, maxdeg, fam, fa, fb, BLOCKED_I32, BLOCKED_F32, BLOCKED_SCALARS)
    assert (py is None) == (nat is None)
    if py is None:
        return
    for name in BLOCKED_I32:
        np.testing.assert_array_equal(nat[name], np.asarray(py[name], dtype=np.int32).ravel(), err_msg=name)
    for name in BLOCKED_F32:
        np.testing.assert_array_equal(nat[name], np.asarray(py[name], dtype=np.float32).ravel(), err_msg=name)
    for name in BLOCKED_SCALARS:
        assert nat[name] == float(py[name]), name


PP_I32 = ("node_seg", "cold_seg", "block_seg", "blk_dims", "blk_run", "hot_dim", "hot_deg", "hot_soff", "node",
          "cold", "run")
PP_F32 = ("blk_ab", "cold_ab", "node_c", "coef")
PP_SCALARS = ("dstride", "row", "n_hb", "n_vp", "n_hot_dims", "n_nodes", "n_cold_groups", "max_depth",
              "n_cold_blocks")


@pytest.mark.parametrize("d,t,d_out,fam_id", [(1, 3.0, 1, 0), (3, 4.5, 2, 0), (6, 5.0, 1, 1), (12, 6.0, 5, 0),
                                              (40, 5.5, 1, 0), (60, 5.8, 8, 1), (200, 6.5, 3, 0)])
def test_perpoint_tables_equal(d, t, d_out, fam_id):
    tr, C, maxdeg, fam, fa, fb = _case(d, t, d_out, fam_id, d + d_out)
    py = build_layout(tr, C, maxdeg, d, d_out, fam, fa, fb)
    nat = _capi.host_layout("perpoint", tr, C, d_out, maxdeg, fam, fa, fb, PP_I32, PP_F32, PP_SCALARS)
    for name in PP_I32:
        np.testing.assert_array_equal(nat[name], np.asarray(py[name], dtype=np.int32).ravel(), err_msg=name)
    for name in PP_F32:
        np.testing.assert_array_equal(nat[name], np.asarray(py[name], dtype=np.float32).ravel(), err_msg=name)
    for name in PP_SCALARS:
        assert nat[name] == float(py[name]), name


P64_I32 = ("node_seg", "cold_seg", "hot_dim", "hot_deg", "hot_soff", "node", "cold", "run")
P64_F64 = ("node_c", "cold_ab", "terms", "coef")
P64_SCALARS = ("d_out", "dstride", "row", "n_hb", "n_vp", "n_hot_dims", "n_nodes", "n_cold_groups", "max_depth",
               "n_terms")


@pytest.mark.parametrize("d,t,fam_id,unit,d_out", [(1, 3.0, 0, True, 1), (6, 5.0, 1, False, 1), (40, 5.5, 0, True, 1),
                                                   (12, 6.0, 1, False, 5), (60, 5.8, 0, True, 8),
                                                   (200, 6.5, 0, False, 1), (1000, 8.22452, 0, True, 1)])
def test_fp64_tables_equal(d, t, fam_id, unit, d_out):
    """The FP64 evaluator's layout (one term per entry): library and package
    builders agree bit for bit, FP64 coefficients included."""
    from smolyax_gb300.spectral import build_layout64

    tr, C, maxdeg, fam, fa, fb = _case(d, t, d_out, fam_id, d + 1)
    if unit:
        fa, fb = np.ones(d), np.zeros(d)
    C = C.astype(np.float64) * (1 + 1e-9 * np.arange(C.size).reshape(C.shape))  # values not representable in FP32
    py = build_layout64(tr, C, maxdeg, d, fam, fa, fb)
    nat = _capi.host_layout("perpoint", tr, C, d_out, maxdeg, fam, fa, fb, P64_I32, P64_F64, P64_SCALARS, fp64=True)
    for name in P64_I32:
        np.testing.assert_array_equal(nat[name], np.asarray(py[name], dtype=np.int32).ravel(), err_msg=name)
    for name in P64_F64:
        a = np.asarray(py[name], dtype=np.float64).ravel()
        assert nat[name].view(np.int64).tolist() == a.view(np.int64).tolist(), name
    for name in P64_SCALARS:
        assert nat[name] == float(py[name]), name


@pytest.mark.parametrize("d,t", [(1, 3.0), (12, 6.0), (200, 6.5), (1000, 8.22452)])
def test_tape_equal(d, t):
    tr, C, maxdeg, fam, fa, fb = _case(d, t, 1, 0, 1)
    py = build_tape(tr, maxdeg)
    nat = _capi.host_layout("tape", tr, None, 1, maxdeg, fam, fa, fb, ("dims", "dmax", "dsoff", "tape", "ent", "lvl1"),
                            (), ("n_slots", "K", "ldk"))
    for name in ("dims", "dmax", "dsoff", "tape", "ent", "lvl1"):
        np.testing.assert_array_equal(nat[name], np.asarray(py[name]).astype(np.int32), err_msg=name)
    assert nat["n_slots"] == py["n_slots"] and nat["K"] == py["ent"].size
