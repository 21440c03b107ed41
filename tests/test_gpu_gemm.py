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


WS_SHAPES = [(128, 128, 64), (130, 257, 64), (1000, 300, 256), (300, 1000, 100), (4096, 4096, 256), (513, 129, 1),
             (7, 5, 3), (2000, 33, 256), (33, 2000, 128), (8192, 2048, 256), (996, 130, 256), (4, 4, 4)]


@pytest.mark.parametrize("m,n,k", WS_SHAPES)
@pytest.mark.parametrize("tiles", [0, 1, 3])
@pytest.mark.parametrize("pad", [0, 4, 1])
def test_sgemm_bf16x3_warp_specialised_matches_one_tile_kernel(gpu, m, n, k, tiles, pad):
    """The multi-tile warp-specialised update issues the same tensor-core
    products in the same order as the one-tile-per-CTA kernel, so C is
    bitwise the same, for any number of tiles per CTA, ragged edges and a
    padded leading dimension: ldc = m rounded up to a multiple of 4, plus 0
    or 4 (the TMA store needs 16-byte column strides), or plus 1, where the
    library falls back to the one-tile kernel (as it does for m not a
    multiple of 4, whose last 16-byte unit of a column holds rows after m);
    the rows between m and ldc must come back untouched either way."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(m * 5 + n * 11 + k)
    ldc = (m + 3) // 4 * 4 + pad
    A = _cm(torch.randn(m, k, device="cuda", generator=g, dtype=torch.float32))
    B = _cm(torch.randn(k, n, device="cuda", generator=g, dtype=torch.float32))
    Cbuf = torch.randn(n, ldc, device="cuda", generator=g, dtype=torch.float32)   # column-major, ld = ldc
    L = gpu.lib()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = []
    for ws in (0, 1):
        old_ws, old_t = gpu.set_option("gemm_ws", ws), gpu.set_option("gemm_tiles", tiles)
        try:
            C = Cbuf.clone()
            rc = L.gb300_sgemm_update_dev(0, m, n, k, ctypes.c_void_p(A.data_ptr()), m, ctypes.c_void_p(B.data_ptr()),
                                          k, ctypes.c_void_p(C.data_ptr()), ldc, s)
            assert rc == 0
            torch.cuda.synchronize()
            outs.append(C)
        finally:
            gpu.set_option("gemm_ws", old_ws)
            gpu.set_option("gemm_tiles", old_t)
    assert torch.equal(outs[0], outs[1])
    assert torch.equal(outs[1][:, m:], Cbuf[:, m:])           # rows beyond m untouched
    ref = Cbuf[:, :m].double().t() - A.double() @ B.double()
    mag = A.double().abs() @ B.double().abs() + Cbuf[:, :m].double().t().abs()
    err = (outs[1][:, :m].double().t() - ref).abs()
    tol = 2.0 ** -14 * mag + (k + 2) * 2.0 ** -24 * mag + 1e-30
    assert bool((err <= tol).all())
