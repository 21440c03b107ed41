"""The adjoint of X = A^{-1} B from the stored LU factors and IPIV:
gB = A^{-T} gX (the transposed solve), gA = -gB X^T (rank-nrhs update).

Checked against a gradient built from the oracle's DGETRS('T')
(SRC/dgetrs.f:199-217) on the same factors and DGEMM('N','T'), against
central finite differences with h = 1e-6, with torch.autograd.gradcheck,
and on the 64 x (n = 2048, nrhs = 8) batch.
"""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _system(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n)) / np.sqrt(n) + np.eye(n)
    b = rng.standard_normal((n, nrhs))
    gx = rng.standard_normal((n, nrhs))
    return a, b, gx


def _forward(gpu, a, b):
    import torch
    LU = gpu.to_colmajor(a)
    ip = torch.empty(a.shape[0], dtype=torch.int32, device="cuda")
    assert gpu.getrf_dev(LU, ip) == 0
    X = gpu.to_colmajor(b)
    gpu.getrs_dev(LU, ip, X)
    return LU, ip, X


def _oracle_dgemm_nt(gb, x):
    """-gB X^T with the oracle's reference DGEMM('N','T', -1, gB, X, 0, C)."""
    n, k = gb.shape
    gb = np.asfortranarray(gb)
    x = np.asfortranarray(x)
    c = np.zeros((n, n), order="F")
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    oracle.lib().or_dgemm(b"N", b"T", n, n, k, -1.0, p(gb), n, p(x), n, 0.0, p(c), n)
    return c


@pytest.mark.parametrize("n,nrhs", [(1, 1), (37, 3), (300, 5), (1024, 8)])
def test_adjoint_matches_reference_getrs_T(gpu, n, nrhs):
    a, b, gx = _system(n, nrhs, n)
    LU, ip, X = _forward(gpu, a, b)
    gB, gA = gpu.adjoint_dev(LU, ip, X, gpu.to_colmajor(gx))
    lu_h, ip_h, x_h = LU.cpu().numpy(), ip.cpu().numpy(), X.cpu().numpy()
    gb_ref, info = oracle.getrs(lu_h, ip_h, gx, "T")
    assert info == 0
    scale = np.abs(gb_ref).max() * n * 2.0 ** -52 * 1e3
    assert np.abs(gB.cpu().numpy() - gb_ref).max() <= scale
    ga_ref = _oracle_dgemm_nt(gb_ref, x_h)
    assert np.abs(gA.cpu().numpy() - ga_ref).max() <= np.abs(ga_ref).max() * 1e-10 + 1e-300


def test_adjoint_rank_update_exact(gpu, exact_mode):
    a, b, gx = _system(200, 6, 3)
    LU, ip, X = _forward(gpu, a, b)
    gB, gA = gpu.adjoint_dev(LU, ip, X, gpu.to_colmajor(gx))
    ga_ref = _oracle_dgemm_nt(gB.cpu().numpy(), X.cpu().numpy())
    assert gA.cpu().numpy().tobytes(order="F") == np.asfortranarray(ga_ref).tobytes(order="F")


def test_adjoint_central_differences(gpu):
    """d/dA and d/dB of L = sum(gX * X(A, B)) at sampled entries, h = 1e-6."""
    n, nrhs, h = 40, 3, 1e-6
    a, b, gx = _system(n, nrhs, 11)

    def loss(aa, bb):
        _, _, x, info = gpu.gesv(aa, bb)
        assert info == 0
        return float(np.sum(gx * x))

    LU, ip, X = _forward(gpu, a, b)
    gB, gA = gpu.adjoint_dev(LU, ip, X, gpu.to_colmajor(gx))
    gA, gB = gA.cpu().numpy(), gB.cpu().numpy()
    rng = np.random.default_rng(5)
    for _ in range(12):
        i, j = rng.integers(0, n, 2)
        ap, am = a.copy(), a.copy()
        ap[i, j] += h
        am[i, j] -= h
        fd = (loss(ap, b) - loss(am, b)) / (2 * h)
        assert abs(fd - gA[i, j]) <= 1e-6 * max(1.0, abs(gA[i, j])), (i, j, fd, gA[i, j])
    for _ in range(6):
        i, q = rng.integers(0, n), rng.integers(0, nrhs)
        bp, bm = b.copy(), b.copy()
        bp[i, q] += h
        bm[i, q] -= h
        fd = (loss(a, bp) - loss(a, bm)) / (2 * h)
        assert abs(fd - gB[i, q]) <= 1e-6 * max(1.0, abs(gB[i, q]))


def test_autograd_gradcheck(gpu):
    import torch
    g = torch.Generator(device="cuda").manual_seed(0)
    A = (torch.randn(6, 6, dtype=torch.float64, device="cuda", generator=g) + 3 * torch.eye(6, dtype=torch.float64,
                                                                                          device="cuda"))
    B = torch.randn(6, 2, dtype=torch.float64, device="cuda", generator=g)
    A.requires_grad_(True)
    B.requires_grad_(True)
    assert torch.autograd.gradcheck(gpu.solve, (A, B), eps=1e-6, atol=1e-7, rtol=1e-6)


def test_adjoint_batch_64x2048(gpu):
    """The differentiable batched case: 64 systems of n = 2048,
    A = N(0,1)/sqrt(n) + I, B and gX of 8 columns."""
    import torch
    batch, n, nrhs = 64, 2048, 8
    g = torch.Generator(device="cuda").manual_seed(1)
    LU = torch.randn(batch, n, n, dtype=torch.float64, device="cuda", generator=g) / n ** 0.5
    LU += torch.eye(n, dtype=torch.float64, device="cuda")
    A0 = LU.clone()
    X = torch.randn(batch, nrhs, n, dtype=torch.float64, device="cuda", generator=g)   # column-major n x nrhs each
    B0 = X.clone()
    GX = torch.randn(batch, nrhs, n, dtype=torch.float64, device="cuda", generator=g)
    ip = torch.empty(batch, n, dtype=torch.int32, device="cuda")
    L = gpu.lib()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    info = ctypes.c_int(0)
    vp = ctypes.c_void_p
    for k in range(batch):
        # the (n, n) slice is read as column-major: A_k^T of the row-major storage; it is still A + noise
        assert L.gb300_dgesv_dev(n, nrhs, vp(LU[k].data_ptr()), n, vp(ip[k].data_ptr()), vp(X[k].data_ptr()), n,
                                 ctypes.byref(info), s) == 0 and info.value == 0
    GB = torch.empty_like(GX)
    GA = torch.empty_like(LU)
    rc = L.gb300_dgesv_adjoint_batched_dev(batch, n, nrhs, vp(LU.data_ptr()), n * n, vp(ip.data_ptr()), n,
                                           vp(X.data_ptr()), n * nrhs, vp(GX.data_ptr()), n * nrhs,
                                           vp(GB.data_ptr()), n * nrhs, vp(GA.data_ptr()), n * n, s)
    assert rc == 0
    for k in (0, 1, 31, batch - 1):
        lu_h = LU[k].cpu().numpy().T            # column-major view of the packed factors
        ip_h = ip[k].cpu().numpy()
        gx_h = GX[k].cpu().numpy().T
        gb_ref, info_r = oracle.getrs(np.asfortranarray(lu_h), ip_h, gx_h, "T")
        gb_gpu = GB[k].cpu().numpy().T
        assert np.abs(gb_gpu - gb_ref).max() <= np.abs(gb_ref).max() * 1e-10
        ga_ref = _oracle_dgemm_nt(gb_ref, X[k].cpu().numpy().T)
        assert np.abs(GA[k].cpu().numpy().T - ga_ref).max() <= np.abs(ga_ref).max() * 1e-10
        # the solve itself: A X = B
        a_h = A0[k].cpu().numpy().T
        assert np.abs(a_h @ X[k].cpu().numpy().T - B0[k].cpu().numpy().T).max() < 1e-10


@pytest.mark.parametrize("n,nrhs,batch", [(100, 3, 5), (129, 1, 3), (64, 16, 2)])
def test_adjoint_batched_ragged_all_systems(gpu, n, nrhs, batch):
    """Batched adjoint at sizes off the 64-row blocks: every system's gB
    and gA against the oracle's DGETRS('T') and DGEMM."""
    import torch
    rng = np.random.default_rng(n + nrhs)
    a = rng.standard_normal((batch, n, n)) + 3 * np.eye(n)
    lus, ips = [], []
    for k in range(batch):
        lu, ip, info = oracle.getrf(np.asfortranarray(a[k]))
        assert info == 0
        lus.append(lu)
        ips.append(ip)
    x = rng.standard_normal((batch, n, nrhs))
    gx = rng.standard_normal((batch, n, nrhs))
    # device copies, column-major per system (stored as the transpose of a row-major (cols, rows) array)
    LU = torch.from_numpy(np.stack([l.T for l in lus])).cuda().contiguous()
    IP = torch.from_numpy(np.stack(ips).astype(np.int32)).cuda().contiguous()
    X = torch.from_numpy(np.ascontiguousarray(np.transpose(x, (0, 2, 1)))).cuda()
    GX = torch.from_numpy(np.ascontiguousarray(np.transpose(gx, (0, 2, 1)))).cuda()
    GB = torch.empty_like(GX)
    GA = torch.empty_like(LU)
    L = gpu.lib()
    vp = ctypes.c_void_p
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.gb300_dgesv_adjoint_batched_dev(batch, n, nrhs, vp(LU.data_ptr()), n * n, vp(IP.data_ptr()), n,
                                           vp(X.data_ptr()), n * nrhs, vp(GX.data_ptr()), n * nrhs,
                                           vp(GB.data_ptr()), n * nrhs, vp(GA.data_ptr()), n * n, s)
    assert rc == 0
    for k in range(batch):
        gb_ref, _ = oracle.getrs(lus[k], ips[k], gx[k], "T")
        gb_gpu = GB[k].cpu().numpy().T
        assert np.abs(gb_gpu - gb_ref).max() <= np.abs(gb_ref).max() * 1e-11
        ga_ref = _oracle_dgemm_nt(gb_ref, x[k])
        assert np.abs(GA[k].cpu().numpy().T - ga_ref).max() <= np.abs(ga_ref).max() * 1e-11
