"""The FP64 DGESV configuration at full size (n = 16384, nrhs = 16, A iid
U[-1,1] by DLARNV idist 2, B iid N(0,1) drawn next; SRC/dgesv.f:148-173),
too large for the oracle to factor in seconds, checked by properties that do
not depend on the size:

  * INFO = 0 and IPIV a valid pivot sequence (1 <= IPIV(i) <= n, IPIV(i) >= i);
  * IPIV(1) is the IDAMAX of the first column (BLAS/SRC/idamax.f:93-123);
  * partial pivoting: every |L(i,j)| <= 1 (SRC/dgetrf2.f:192-214);
  * the DGET02 ratio ||B - A X||_1 / (||A||_1 ||X||_1 eps) of every
    right-hand side (TESTING/LIN/dget02.f:176-219), computed on the GPU in
    FP64, below sqrt(n) (the reference's size-aware rule for large systems,
    TESTING/LIN/ddrvab.f:362-365; its THRESH = 30 is set for n <= 50), and
    within 4x of the ratio of an independent FP64 solve (torch.linalg.solve)
    of the same system.
"""
import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu


def test_dgesv_fp64_n16384_nrhs16(gpu):
    import torch
    n, nrhs = 16384, 16
    a, b = oracle.config_dgesv_fp64(n, nrhs, 1)
    lu, ip, x, info = gpu.gesv(a, b)
    assert info == 0
    ip = np.asarray(ip)
    assert ip.min() >= 1 and ip.max() <= n
    assert np.all(ip >= np.arange(1, n + 1))
    assert ip[0] == 1 + int(np.argmax(np.abs(a[:, 0])))
    dev = torch.device("cuda")
    LU = torch.from_numpy(np.ascontiguousarray(lu.T)).to(dev)       # row i of LU^T = column i of LU
    strict_lower = torch.tril(torch.ones(n, n, dtype=torch.bool, device=dev), diagonal=-1).t()
    assert LU.abs().masked_select(strict_lower).max().item() <= 1.0
    del LU, strict_lower
    A = torch.from_numpy(np.ascontiguousarray(a.T)).to(dev).t()
    X = torch.from_numpy(np.ascontiguousarray(x.T)).to(dev).t()
    B = torch.from_numpy(np.ascontiguousarray(b.T)).to(dev).t()
    anorm = A.abs().sum(dim=0).max().item()

    def ratios(Xs):
        R = B - A @ Xs
        return [R[:, j].abs().sum().item() / (anorm * Xs[:, j].abs().sum().item() * ck.EPS64) for j in range(nrhs)]

    ours = ratios(X)
    ref = ratios(torch.linalg.solve(A, B))
    for j in range(nrhs):
        assert ours[j] < np.sqrt(n), (j, ours[j])
        assert ours[j] <= 4.0 * max(ref[j], 1.0), (j, ours[j], ref[j])
