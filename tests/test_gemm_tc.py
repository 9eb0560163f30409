"""Tensor-core GEMM (tcgen05) of the learned tool predictor against float64
numpy on the same bf16 inputs."""

import ctypes

import numpy as np
import pytest

from blademaster_gb300 import _native

pytestmark = pytest.mark.gpu


def bf16(x):
    """Round float32 to bfloat16 (nearest even), returned as (uint16 bits, float64 values)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return rounded, (rounded.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def gemm(a_bits, b_bits, M, N, K, bias=None, relu=False):
    import torch

    dev = "cuda:0"
    A = torch.as_tensor(a_bits.view(np.int16), device=dev)
    B = torch.as_tensor(b_bits.view(np.int16), device=dev)
    D = torch.zeros(M, N, dtype=torch.float32, device=dev)
    Dh = torch.zeros(M, N, dtype=torch.int16, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    bias_t = torch.as_tensor(bias, dtype=torch.float32, device=dev) if bias is not None else None
    lib = _native.lib()
    _native.check(lib.bm_gemm_tn_bf16(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
                                      ctypes.c_void_p(D.data_ptr()), M, N, K,
                                      ctypes.c_void_p(bias_t.data_ptr()) if bias_t is not None else None, int(relu),
                                      ctypes.c_void_p(Dh.data_ptr()), ctypes.c_void_p(status.data_ptr()), None))
    torch.cuda.synchronize()
    assert status.item() == 0
    return D.cpu().numpy(), Dh.cpu().numpy().view(np.uint16)


@pytest.mark.parametrize("M,N,K", [(128, 16, 32), (128, 256, 96), (300, 64, 256), (256, 256, 512)])
def test_gemm_matches_float64(M, N, K):
    rng = np.random.default_rng(M + N + K)
    a_bits, a = bf16(rng.normal(size=(M, K)))
    b_bits, b = bf16(rng.normal(size=(N, K)))
    D, _ = gemm(a_bits, b_bits, M, N, K)
    expected = a @ b.T
    np.testing.assert_allclose(D, expected, rtol=1e-5, atol=1e-4 * np.sqrt(K))


def test_gemm_bias_relu_and_bf16_copy():
    rng = np.random.default_rng(7)
    M, N, K = 256, 32, 64
    a_bits, a = bf16(rng.normal(size=(M, K)))
    b_bits, b = bf16(rng.normal(size=(N, K)))
    bias = rng.normal(size=N).astype(np.float32)
    D, Dh = gemm(a_bits, b_bits, M, N, K, bias=bias, relu=True)
    expected = np.maximum(a @ b.T + bias, 0.0)
    np.testing.assert_allclose(D, expected, rtol=1e-5, atol=1e-4 * np.sqrt(K))
    np.testing.assert_array_equal(Dh, bf16(D)[0])


def test_gemm_wait_timeout_reports_status_and_returns():
    """The bounded-wait path: with the K loop's poll limit at 0 the first wait
    for a stage (chunk 4 of 8 reuses chunk 0's stage) gives up at once; the
    kernel drains the MMAs in flight with the full limit, records status 1,
    writes nothing and returns.  The default limit then computes normally."""
    import torch

    rng = np.random.default_rng(3)
    M, N, K = 128, 64, 256
    a_bits, a = bf16(rng.normal(size=(M, K)))
    b_bits, b = bf16(rng.normal(size=(N, K)))
    dev = "cuda:0"
    A = torch.as_tensor(a_bits.view(np.int16), device=dev)
    B = torch.as_tensor(b_bits.view(np.int16), device=dev)
    D = torch.zeros(M, N, dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    lib = _native.lib()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    _native.check(lib.bm_gemm_set_loop_wait_limit(0))
    try:
        _native.check(lib.bm_gemm_tn_bf16(p(A), p(B), p(D), M, N, K, None, 0, None, p(status), None))
        torch.cuda.synchronize()
    finally:
        _native.check(lib.bm_gemm_set_loop_wait_limit(-1))
    assert status.item() == 1
    assert not D.any()
    status.zero_()
    _native.check(lib.bm_gemm_tn_bf16(p(A), p(B), p(D), M, N, K, None, 0, None, p(status), None))
    torch.cuda.synchronize()
    assert status.item() == 0
    np.testing.assert_allclose(D.cpu().numpy(), a @ b.T, rtol=1e-5, atol=1e-4 * np.sqrt(K))
