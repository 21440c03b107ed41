"""The allocation-free DGETRS entry point (gb300_dgetrs_noalloc).

Some callers cannot allocate GPU memory when they solve: a process that
reserved its whole device budget up front, a latency-critical loop, code in
an allocator callback.  gb300_dgetrs_noalloc serves them from a fixed
scratch array inside the library.  This file is collected last on purpose,
so that a run stopping at the first failure has already run every other
test; it passes alone in a fresh process and after the other tests.

Checked through the C ABI: two calls in a row give the same solution as the
allocating gb300_dgetrs_dev (both transposes), within the test tolerance of
the other GETRS tests, and sizes beyond the fixed scratch are refused.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(gpu, n, nrhs, seed):
    """A random system and its LU factors computed on the GPU (both solves
    under comparison use the same factors)."""
    import torch
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n))
    b = rng.standard_normal((n, nrhs))
    dA = gpu.to_colmajor(a)
    dIp = torch.empty(n, dtype=torch.int32, device="cuda")
    assert gpu.getrf_dev(dA, dIp) == 0
    return a, b, dA, dIp


def _call(L, fn, trans, dA, dIp, dB):
    import torch
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    n, nrhs = dB.shape
    return fn(ctypes.c_char(trans.encode()), n, nrhs, ctypes.c_void_p(dA.data_ptr()), dA.stride(1),
              ctypes.c_void_p(dIp.data_ptr()), ctypes.c_void_p(dB.data_ptr()), dB.stride(1) if nrhs > 1 else n, s)


@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,nrhs", [(1, 1), (300, 3), (2048, 8), (16384, 1)])
def test_noalloc_matches_allocating_getrs(gpu, trans, n, nrhs):
    L = gpu.lib()
    L.gb300_dgetrs_noalloc.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    a, b, dA, dIp = _setup(gpu, n, nrhs, 40 + n)
    ref = gpu.to_colmajor(b)
    assert _call(L, L.gb300_dgetrs_dev, trans, dA, dIp, ref) == 0
    x_ref = ref.cpu().numpy()
    for _ in range(2):                       # two calls in a row share the scratch array
        dB = gpu.to_colmajor(b)
        assert _call(L, L.gb300_dgetrs_noalloc, trans, dA, dIp, dB) == 0
        x = dB.cpu().numpy()
        tol = np.abs(x_ref).max() * n * np.finfo(np.float64).eps * 1e3
        assert np.abs(x - x_ref).max() <= tol


@pytest.mark.parametrize("trans,n,nrhs,pad", [("C", 8192, 16, 3), ("N", 4096, 32, 5), ("T", 16384, 8, 0)])
def test_noalloc_at_scratch_limit_with_padded_ldb(gpu, trans, n, nrhs, pad):
    """n*nrhs exactly at the 131072-element limit, ldb > n, TRANS = 'C':
    the fixed offsets inside the scratch array at their largest extent.
    Checked against the allocating entry point and, through the residual,
    against the system itself."""
    import torch
    L = gpu.lib()
    L.gb300_dgetrs_noalloc.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    a, b, dA, dIp = _setup(gpu, n, nrhs, 70 + n)
    ldb = n + pad
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def padded():
        buf = torch.zeros((nrhs, ldb), dtype=torch.float64, device="cuda")
        buf[:, :n] = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
        return buf

    def run(fn, buf):
        return fn(ctypes.c_char(trans.encode()), n, nrhs, ctypes.c_void_p(dA.data_ptr()), dA.stride(1),
                  ctypes.c_void_p(dIp.data_ptr()), ctypes.c_void_p(buf.data_ptr()), ldb, s)

    ref = padded()
    assert run(L.gb300_dgetrs_dev, ref) == 0
    x_ref = ref[:, :n].cpu().numpy().T
    for _ in range(2):
        buf = padded()
        assert run(L.gb300_dgetrs_noalloc, buf) == 0
        got = buf.cpu().numpy()
        assert np.all(got[:, n:] == 0.0)                   # the padding rows are not written
        x = got[:, :n].T
        tol = np.abs(x_ref).max() * n * np.finfo(np.float64).eps * 1e3
        assert np.abs(x - x_ref).max() <= tol
        op = a if trans == "N" else a.T
        r = np.abs(b - op @ x).max() / (np.abs(op).sum(axis=1).max() * np.abs(x).max() * n * np.finfo(float).eps)
        assert r < 30.0


def test_noalloc_rejects_sizes_beyond_scratch(gpu):
    import torch
    L = gpu.lib()
    L.gb300_dgetrs_noalloc.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # n above the limit, and n*nrhs above the limit: refused before any device work
    assert L.gb300_dgetrs_noalloc(b"N", 16385, 1, None, 16385, None, None, 16385, s) == -100
    assert L.gb300_dgetrs_noalloc(b"N", 8192, 17, None, 8192, None, None, 8192, s) == -100
