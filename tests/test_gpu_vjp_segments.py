"""The gradient walk in tape segments (``csrc/spectral.cu`` vjp_rows / vjp_seg /
vjp_sum kernels).  For a plan with a long tape (|Lambda| ~ 1.3e4, so the walk
is cut into segments at depth-1 entries, one warp per 32 points and segment,
each with its own adjoint copy):

* dL/dx equals the single-walk result (the same plan with one segment) within
  the FP32 rounding of the adjoint sums: 2^-16 of the scale;
* a point's dL/dx does not depend on the batch it comes in (bit-identical
  alone and within a larger call: the segments are fixed per plan);
* dL/dx agrees with the FP64 Jacobian of the interpolant contracted with the
  cotangent, at 1e-5 of the scale (the FP32 form's bound).
"""
import numpy as np
import pytest
import torch

import functions as fns

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plan():
    from smolyax_gb300 import SmolyakBarycentricInterpolator, indices, nodes

    d, d_out = 24, 3
    k = np.log((2 + np.arange(d)) / np.log(2))
    t = indices.find_approximate_threshold(k, 13000, nested=True, accuracy=0.01)
    ip = SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=d), k=k, t=t, d_out=d_out,
                                        f=fns.rational_vec(d, d_out, seed=5))
    sp = ip.spectral_plan()
    ops = sp._backward_ops()
    assert ops["vjp_seg"][1] >= 3, ops["vjp_seg"][1]
    return ip, sp, ops


def test_segments_match_single_walk_and_jacobian(plan):
    ip, sp, ops = plan
    rng = np.random.default_rng(0)
    P = 300
    x = torch.as_tensor(rng.uniform(-1, 1, (P, ip.d_in)), device="cuda")
    g = torch.as_tensor(rng.normal(size=(P, ip.d_out)).astype(np.float32), device="cuda")
    dx_seg, _ = sp.vjp(x, g, need_x=True, need_coef=False)
    kept = ops["vjp_seg"]
    try:
        ops["vjp_seg"] = (None, 1)
        dx_one, _ = sp.vjp(x, g, need_x=True, need_coef=False)
    finally:
        ops["vjp_seg"] = kept
    scale = float(dx_one.abs().max())
    diff = float((dx_seg - dx_one).abs().max())
    J = ip.gradient(x)  # [P, d_out, d_in] FP64
    ref = torch.einsum("po,poi->pi", g.double(), J)
    err = float((dx_seg - ref).abs().max()) / float(ref.abs().max())
    print("segments %d: vs single walk %.3e of scale, vs FP64 Jacobian %.3e" % (kept[1], diff / scale, err))
    assert diff <= 2.0**-16 * scale
    assert err < 1e-5


def test_result_independent_of_batch(plan):
    ip, sp, ops = plan
    rng = np.random.default_rng(1)
    x = torch.as_tensor(rng.uniform(-1, 1, (1000, ip.d_in)), device="cuda")
    g = torch.ones(1000, ip.d_out, dtype=torch.float32, device="cuda")
    big, _ = sp.vjp(x, g, need_x=True, need_coef=False)
    small, _ = sp.vjp(x[:37].contiguous(), g[:37].contiguous(), need_x=True, need_coef=False)
    assert torch.equal(big[:37], small)
