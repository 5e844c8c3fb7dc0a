"""tcgen05 3xTF32 contraction (``smx_gemm_tf32x3``) against an FP64 product.

Bound: norm-wise relative error 2e-6 for K up to 5000 (hi + lo keeps ~22 bits of
each operand; the tensor cores accumulate in FP32 with truncation, in chunks of
64 products that are added in registers; measured 4e-7 .. 8e-7 at every K).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(A, B, bias=None):
    import torch

    from smolyax_gb300 import _capi

    dev = torch.device("cuda", torch.cuda.current_device())
    M, K = A.shape
    N = B.shape[0]
    ld = (K + 3) // 4 * 4
    st = _capi.stream_ptr(torch.cuda.current_stream())

    def split(X):
        Xd = torch.zeros(X.shape[0], ld, dtype=torch.float32, device=dev)
        Xd[:, :K] = torch.as_tensor(X, dtype=torch.float32)
        hi = torch.zeros_like(Xd)
        lo = torch.zeros_like(Xd)
        _capi.call("smx_split_tf32", _capi.ptr(Xd), X.shape[0], ld, ld, _capi.ptr(hi), _capi.ptr(lo), ld, st)
        return hi, lo

    Ah, Al = split(A)
    Bh, Bl = split(B)
    D = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    b = None if bias is None else torch.as_tensor(bias, dtype=torch.float32, device=dev)
    _capi.call("smx_gemm_tf32x3", _capi.ptr(Ah), _capi.ptr(Al), ld, _capi.ptr(Bh), _capi.ptr(Bl), ld, M, N, K,
               _capi.ptr(D), N, _capi.ptr(b), 0, _capi.ptr(err), st)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return D.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (300, 200, 100), (256, 256, 1000), (1000, 64, 5000), (77, 520, 40)])
def test_gemm_tf32x3(M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = rng.normal(size=(N, K)).astype(np.float32)
    bias = rng.normal(size=N).astype(np.float32)
    D = _gemm(A, B, bias)
    ref = A.astype(np.float64) @ B.astype(np.float64).T + bias
    err = np.max(np.abs(D - ref)) / np.max(np.abs(ref))
    print("M=%d N=%d K=%d norm-wise rel err %.2e" % (M, N, K, err))
    assert err < 2e-6


def _gemm_bf16(A, B, bias=None):
    import torch

    from smolyax_gb300 import _capi

    dev = torch.device("cuda", torch.cuda.current_device())
    M, K = A.shape
    N = B.shape[0]
    ld = (K + 7) // 8 * 8  # BF16 rows: 16-byte pitch for the tensor maps
    st = _capi.stream_ptr(torch.cuda.current_stream())

    def split(X):
        Xd = torch.zeros(X.shape[0], ld, dtype=torch.float32, device=dev)
        Xd[:, :K] = torch.as_tensor(X, dtype=torch.float32)
        hi = torch.zeros(X.shape[0], ld, dtype=torch.bfloat16, device=dev)
        lo = torch.zeros_like(hi)
        _capi.call("smx_split_bf16", _capi.ptr(Xd), X.shape[0], ld, ld, _capi.ptr(hi), _capi.ptr(lo), ld, st)
        return Xd, hi, lo

    Ad, Ah, Al = split(A)
    Bd, Bh, Bl = split(B)
    # the split is hi = round-to-nearest BF16 of x, lo = BF16 of the remainder
    assert torch.equal(Ah, Ad.to(torch.bfloat16))
    assert torch.equal(Al, (Ad - Ah.float()).to(torch.bfloat16))
    D = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    b = None if bias is None else torch.as_tensor(bias, dtype=torch.float32, device=dev)
    _capi.call("smx_gemm_bf16x3", _capi.ptr(Ah), _capi.ptr(Al), ld, _capi.ptr(Bh), _capi.ptr(Bl), ld, M, N, K,
               _capi.ptr(D), N, _capi.ptr(b), 0, _capi.ptr(err), st)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    # the three products the kernel forms, in FP64: hi.hi + hi.lo + lo.hi
    h = lambda t: t.double().cpu().numpy()  # noqa: E731
    ref3 = (h(Ah) @ h(Bh).T + h(Ah) @ h(Bl).T + h(Al) @ h(Bh).T)[:, :N]
    if bias is not None:
        ref3 = ref3 + bias
    return D.cpu().numpy().astype(np.float64), ref3


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 200, 100), (256, 256, 1000), (1000, 64, 5000), (77, 520, 41)])
def test_gemm_bf16x3(M, N, K):
    """Split-BF16 contraction: three BF16 products accumulated in FP32 in tensor
    memory.  Against the FP64 product of the FP32 operands the error is that of
    the 16-bit split (lo.lo dropped, lo rounded): norm-wise bound 1e-4; against
    the FP64 value of the same three products it is FP32 accumulation only."""
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = rng.normal(size=(N, K)).astype(np.float32)
    bias = rng.normal(size=N).astype(np.float32)
    D, ref3 = _gemm_bf16(A, B, bias)
    ref = A.astype(np.float64) @ B.astype(np.float64).T + bias
    scale = np.max(np.abs(ref))
    err = np.max(np.abs(D - ref)) / scale
    err3 = np.max(np.abs(D - ref3)) / scale
    print("M=%d N=%d K=%d bf16x3 norm-wise rel err %.2e (vs its own three products %.2e)" % (M, N, K, err, err3))
    assert err3 < 2e-6
    assert err < 1e-4


@pytest.mark.parametrize("M,N,K,splits", [(1000, 64, 20000, 8), (333, 66, 5000, 5), (130, 7, 999, 3), (256, 128, 64, 4)])
def test_gemm_tf32x3_splitk(M, N, K, splits):
    """Split-K contraction: slices of the K range run side by side and are added in
    slice order, with bias and accumulate; same bound as the unsplit product."""
    import torch

    from smolyax_gb300 import _capi

    dev = torch.device("cuda", torch.cuda.current_device())
    rng = np.random.default_rng(M + N + K + splits)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = rng.normal(size=(N, K)).astype(np.float32)
    bias = rng.normal(size=N).astype(np.float32)
    D0 = rng.normal(size=(M, N)).astype(np.float32)
    ld = (K + 3) // 4 * 4
    st = _capi.stream_ptr(torch.cuda.current_stream())

    def split(X):
        Xd = torch.zeros(X.shape[0], ld, dtype=torch.float32, device=dev)
        Xd[:, :K] = torch.as_tensor(X, dtype=torch.float32)
        hi, lo = torch.zeros_like(Xd), torch.zeros_like(Xd)
        _capi.call("smx_split_tf32", _capi.ptr(Xd), X.shape[0], ld, ld, _capi.ptr(hi), _capi.ptr(lo), ld, st)
        return hi, lo

    Ah, Al = split(A)
    Bh, Bl = split(B)
    ldd = N + 3  # an odd row pitch: the epilogue's scalar path
    D = torch.zeros(M, ldd, dtype=torch.float32, device=dev)
    D[:, :N] = torch.as_tensor(D0, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    nws = _capi.size("smx_gemm_tf32x3_splitk_workspace", M, N, K, splits)
    ws = torch.empty(max(nws, 1), dtype=torch.uint8, device=dev)
    b = torch.as_tensor(bias, device=dev)
    _capi.call("smx_gemm_tf32x3_splitk", _capi.ptr(Ah), _capi.ptr(Al), ld, _capi.ptr(Bh), _capi.ptr(Bl), ld, M, N, K,
               _capi.ptr(D), ldd, _capi.ptr(b), 1, splits, _capi.ptr(ws), nws, _capi.ptr(err), st)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    got = D[:, :N].cpu().numpy().astype(np.float64)
    ref = A.astype(np.float64) @ B.astype(np.float64).T + bias + D0
    e = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    print("split-K M=%d N=%d K=%d splits=%d: norm-wise rel err %.2e" % (M, N, K, splits, e))
    assert e < 2e-6
    assert torch.all(D[:, N:] == 0)  # the pitch padding is untouched


def test_gemm_timeout_path_reports_and_recovers():
    """Failure detection of the tensor-core contraction: with its copy producer
    switched off, the kernel's first pipeline wait runs out after 1 ms; it must
    record error code 2, leave D untouched and return, and the next ordinary
    contraction on the same context must be correct."""
    import torch

    from smolyax_gb300 import _capi

    dev = torch.device("cuda", torch.cuda.current_device())
    st = _capi.stream_ptr(torch.cuda.current_stream())
    M, N, K = 256, 128, 64
    A = torch.zeros(M, K, dtype=torch.float32, device=dev)
    B = torch.zeros(N, K, dtype=torch.float32, device=dev)
    D = torch.full((M, N), 7.0, dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    _capi.call("smx_gemm_tf32x3_timeout_selftest", _capi.ptr(A), _capi.ptr(A), K, _capi.ptr(B), _capi.ptr(B), K, M, N,
               K, _capi.ptr(D), N, _capi.ptr(err), 1_000_000, st)
    torch.cuda.synchronize()
    assert int(err.item()) == 2
    assert bool((D == 7.0).all())
    rng = np.random.default_rng(5)
    A2 = rng.normal(size=(300, 200)).astype(np.float32)
    B2 = rng.normal(size=(150, 200)).astype(np.float32)
    got = _gemm(A2, B2)
    ref = A2.astype(np.float64) @ B2.astype(np.float64).T
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 2e-6
