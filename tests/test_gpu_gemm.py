"""The trailing-matrix update kernels against an FP64 torch reference.

FP64 (DFMA) and FP32 (FFMA) forms: |C - C_ref| within a few ulps of the
accumulated magnitude.  BF16x3 tensor-core form: every product a*b is
replaced by ah*bh + ah*bl + al*bh (ah = bf16(a), al = bf16(a - ah)), which
drops al*bl and the part of a below 16 significant bits, so the bound is
|C - C_ref| <= 2^-14 * (|A| |B|) + FP32 accumulation (K * 2^-24 * (|A| |B|)).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(128, 128, 64), (130, 257, 64), (1000, 300, 256), (64, 70, 32), (300, 1000, 100), (4096, 4096, 256),
          (513, 129, 1), (7, 5, 3)]


def _cm(t):
    """column-major copy of a (m, n) tensor."""
    return t.t().contiguous().t()


@pytest.mark.parametrize("m,n,k", SHAPES)
@pytest.mark.parametrize("mode", [0, 1])
def test_sgemm_update(gpu, m, n, k, mode):
    import torch
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n * 3 + k)
    A = _cm(torch.randn(m, k, device="cuda", generator=g, dtype=torch.float32))
    B = _cm(torch.randn(k, n, device="cuda", generator=g, dtype=torch.float32))
    C = _cm(torch.randn(m, n, device="cuda", generator=g, dtype=torch.float32))
    ref = C.double() - A.double() @ B.double()
    mag = A.double().abs() @ B.double().abs() + C.double().abs()
    L = gpu.lib()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.gb300_sgemm_update_dev(mode, m, n, k, ctypes.c_void_p(A.data_ptr()), m, ctypes.c_void_p(B.data_ptr()), k,
                                  ctypes.c_void_p(C.data_ptr()), m, s)
    assert rc == 0
    err = (C.double() - ref).abs()
    tol = (2.0 ** -14 if mode == 0 else 2.0 ** -22) * mag + (k + 2) * 2.0 ** -24 * mag + 1e-30
    assert bool((err <= tol).all()), f"max err/tol {(err / tol).max().item()}"


@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (257, 130, 64), (1000, 999, 128), (5, 3, 2)])
def test_dgemm_update(gpu, m, n, k):
    import torch
    g = torch.Generator(device="cuda").manual_seed(m + n + k)
    A = _cm(torch.randn(m, k, device="cuda", generator=g, dtype=torch.float64))
    B = _cm(torch.randn(k, n, device="cuda", generator=g, dtype=torch.float64))
    C = _cm(torch.randn(m, n, device="cuda", generator=g, dtype=torch.float64))
    ref = C - A @ B
    mag = A.abs() @ B.abs() + C.abs()
    L = gpu.lib()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.gb300_dgemm_update_dev(m, n, k, ctypes.c_void_p(A.data_ptr()), m, ctypes.c_void_p(B.data_ptr()), k,
                                  ctypes.c_void_p(C.data_ptr()), m, s)
    assert rc == 0
    assert bool(((C - ref).abs() <= (k + 2) * 2.0 ** -52 * mag).all())
