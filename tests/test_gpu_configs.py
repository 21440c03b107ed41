"""The FP64 DGESV configuration at full size (n = 16384, nrhs = 16, A iid
U[-1,1] by DLARNV idist 2 and B iid N(0,1) drawn next from the stream of
scalar seed 1; SRC/dgesv.f:148-173) against the oracle's DGETRF / DGETRS on
the same matrix.  The oracle takes minutes at this size, so its figures are
cached in tests/golden/dgesv_n16384_nrhs16_seed1.npz (made by
tests/golden/make_config2.py); the test regenerates the inputs and checks
their sha256 against the fixture first.

Criteria (the parity rules of the solve path):
  * IPIV identical to the oracle's wherever the oracle's pivot margin exceeds
    rounding: the first differing pivot, if any, must be a near-tie (relative
    margin below 1e-10), after which the factors are not comparable;
  * L/U agree with the oracle's to max |dLU| <= 64 n eps max|LU| on the
    cached sample LU[::128, ::128] (the factors' own magnitude: U grows
    well past max|A| = 1 at this size), and every column sum within n times
    that;
  * the scaled residual ||b - A x||_inf / (||A||_inf ||x||_inf n eps) and the
    DGET02 ratio (TESTING/LIN/dget02.f:176-219) of every right-hand side at
    or below the oracle's own values on the same system;
  * the solution agrees with the oracle's sampled solution to 1e-8 relative
    (A is well conditioned: kappa ~ n for U[-1,1]).
Plus the size-independent checks: INFO = 0, IPIV a valid pivot sequence,
every |L(i,j)| <= 1 (partial pivoting, SRC/dgetrf2.f:192-214).
"""
import hashlib
import os

import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dgesv_n16384_nrhs16_seed1.npz")


@pytest.fixture(scope="module")
def config2():
    fx = np.load(FIX)
    n, nrhs, seed = int(fx["n"]), int(fx["nrhs"]), int(fx["seed"])
    a, b = oracle.config_dgesv_fp64(n, nrhs, seed)
    assert hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest() == str(fx["sha_a"])
    assert hashlib.sha256(np.asfortranarray(b).tobytes(order="F")).hexdigest() == str(fx["sha_b"])
    return fx, a, b


def test_dgesv_fp64_n16384_nrhs16_against_oracle(gpu, config2):
    import torch
    fx, a, b = config2
    n, nrhs = a.shape[0], b.shape[1]
    lu, ip, x, info = gpu.gesv(a, b)
    assert info == 0
    ip = np.asarray(ip, dtype=np.int32)
    assert ip.min() >= 1 and ip.max() <= n and np.all(ip >= np.arange(1, n + 1))

    # pivots: identical up to a near-tie of the oracle's search
    diff = np.nonzero(ip != fx["ipiv"])[0]
    first = int(diff[0]) if diff.size else n
    if first < n:
        assert fx["margin"][first] < 1e-10, (first, fx["margin"][first])
    else:
        # the factors are comparable: a strided sample and every column sum
        eps = np.finfo(np.float64).eps / 2
        scale = np.abs(lu).max() * n * eps
        st = int(fx["stride"])
        d = np.abs(lu[::st, ::st] - fx["lu_sample"]).max()
        assert d <= 64.0 * scale, (d / scale, np.abs(lu).max())
        dcol = np.abs(lu.sum(axis=0) - fx["colsum"]).max()
        assert dcol <= 64.0 * scale * n, dcol / (scale * n)

    dev = torch.device("cuda")
    LU = torch.from_numpy(np.ascontiguousarray(lu.T)).to(dev)       # row i of LU^T = column i of LU
    strict_lower = torch.tril(torch.ones(n, n, dtype=torch.bool, device=dev), diagonal=-1).t()
    assert LU.abs().masked_select(strict_lower).max().item() <= 1.0
    del LU, strict_lower
    A = torch.from_numpy(np.ascontiguousarray(a.T)).to(dev).t()
    X = torch.from_numpy(np.ascontiguousarray(x.T)).to(dev).t()
    B = torch.from_numpy(np.ascontiguousarray(b.T)).to(dev).t()
    R = B - A @ X
    a_inf = A.abs().sum(dim=1).max().item()
    a_1 = A.abs().sum(dim=0).max().item()
    for j in range(nrhs):
        scaled = R[:, j].abs().max().item() / (a_inf * X[:, j].abs().max().item() * n * ck.EPS64)
        dget02 = R[:, j].abs().sum().item() / (a_1 * X[:, j].abs().sum().item() * ck.EPS64)
        assert scaled <= fx["scaled_residual"][j], (j, scaled, fx["scaled_residual"][j])
        assert dget02 <= fx["dget02"][j], (j, dget02, fx["dget02"][j])
    xs = x[:: int(fx["xstride"])]
    assert np.abs(xs - fx["x_sample"]).max() <= 1e-8 * np.abs(fx["x_sample"]).max()
