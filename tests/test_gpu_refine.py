"""DGERFS on the GPU (SRC/dgerfs.f) against the oracle's restatement.

Exact mode: X, FERR and BERR bitwise equal to the oracle (residual, bound,
solves and the DLACN2 estimator all in the reference order).  Default mode:
the DCHKGE refinement tests (TESTING/LIN/dchkge.f:496-520: DGET04 after
refinement and both DGET07 ratios below THRESH), FERR within a factor of
three of the oracle's estimate, and each column's result independent of
the other columns refined with it."""
import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu
THRESH = 30.0


def _system(n, nrhs, imat, seed, trans):
    a, izero = oracle.ge_test_matrix(n, n, imat, seed)
    assert izero == 0
    lu, ipiv, info = oracle.getrf(a)
    assert info == 0
    xact = oracle.random_matrix(n, nrhs, seed + 1, idist=2)[0]
    op = a if trans == "N" else a.T
    b = op @ xact
    x0, _ = oracle.getrs(lu, ipiv, b, trans)
    return a, lu, ipiv, b, x0, xact


@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("n,nrhs,imat", [(1, 1, 1), (2, 2, 2), (5, 3, 3), (10, 15, 4), (50, 2, 8), (50, 1, 9),
                                         (300, 3, 1), (700, 2, 10)])
def test_gerfs_exact_bitwise(gpu, exact_mode, trans, n, nrhs, imat):
    a, lu, ipiv, b, x0, _ = _system(n, nrhs, imat, 31 + n + imat, trans)
    xr, fr, br, ir = oracle.gerfs(a, lu, ipiv, b, x0, trans)
    xg, fg, bg, ig = gpu.gerfs(a, lu, ipiv, b, x0, trans)
    assert ig == ir == 0
    assert xg.tobytes() == xr.tobytes(), "X not bitwise identical"
    assert bg.tobytes() == br.tobytes(), (bg, br)
    assert fg.tobytes() == fr.tobytes(), (fg, fr)


@pytest.mark.parametrize("imat", range(1, 12))
@pytest.mark.parametrize("trans", ["N", "T"])
def test_gerfs_dchkge_ratios(gpu, imat, trans):
    for n in (3, 10, 50, 200):
        if 5 <= imat <= 7 and n < imat - 4:
            continue
        a, izero = oracle.ge_test_matrix(n, n, imat, 1988 + 8 * n)
        if izero:
            continue
        for nrhs in (1, 2, 15):
            a, lu, ipiv, b, x0, xact = _system(n, nrhs, imat, 1988 + 8 * n, trans)
            op = a if trans == "N" else a.T
            rcond = 1.0 / np.linalg.cond(op, 1)
            x, ferr, berr, info = gpu.gerfs(a, lu, ipiv, b, x0, trans)
            assert info == 0
            assert ck.dget04(x, xact, rcond) < THRESH, (n, imat, nrhs)
            r1, r2 = ck.dget07(a, b, x, xact, ferr, berr, trans)
            assert r1 < THRESH and r2 < THRESH, (n, imat, nrhs, r1, r2)
            _, fr, _, _ = oracle.gerfs(a, lu, ipiv, b, x0, trans)
            assert np.all(ferr <= 3 * fr) and np.all(ferr >= fr / 3), (ferr, fr)   # two runs of an estimator


@pytest.mark.parametrize("trans", ["N", "T"])
def test_gerfs_columns_independent(gpu, trans):
    """70 right-hand sides (more than one launch list of 64 columns): each
    column's X, FERR, BERR equal those of refining that column alone."""
    n, nrhs = 256, 70
    a, lu, ipiv, b, x0, _ = _system(n, nrhs, 1, 77, trans)
    x0 = x0 * (1 + 1e-9 * oracle.random_matrix(n, nrhs, 78, idist=2)[0])   # some columns need more steps
    xa, fa, ba, _ = gpu.gerfs(a, lu, ipiv, b, x0, trans)
    for j in (0, 3, 63, 64, 69):
        xj, fj, bj, _ = gpu.gerfs(a, lu, ipiv, b[:, j:j + 1], x0[:, j:j + 1], trans)
        assert xj[:, 0].tobytes() == xa[:, j].tobytes()
        assert fj[0] == fa[j] and bj[0] == ba[j]


def test_gerfs_device_api_matches_host_abi(gpu):
    import torch
    n, nrhs = 400, 3
    a, lu, ipiv, b, x0, _ = _system(n, nrhs, 2, 5, "N")
    xh, fh, bh, _ = gpu.gerfs(a, lu, ipiv, b, x0, "N")
    A = gpu.to_colmajor(a)
    AF = gpu.to_colmajor(lu)
    B = gpu.to_colmajor(b)
    X = gpu.to_colmajor(x0)
    ip = torch.from_numpy(np.ascontiguousarray(ipiv, dtype=np.int32)).cuda()
    ferr = torch.zeros(nrhs, dtype=torch.float64, device="cuda")
    berr = torch.zeros(nrhs, dtype=torch.float64, device="cuda")
    gpu.gerfs_dev(A, AF, ip, B, X, ferr, berr, "N")
    torch.cuda.synchronize()
    assert X.cpu().numpy().tobytes(order="F") == np.asfortranarray(xh).tobytes(order="F")
    assert np.array_equal(ferr.cpu().numpy(), fh) and np.array_equal(berr.cpu().numpy(), bh)


def test_gerfs_n4096_refines_perturbed_solution(gpu):
    """A perturbed solution of a well-conditioned n=4096 system: refinement
    restores a componentwise backward error of a few eps and a forward
    error bound that holds."""
    n, nrhs = 4096, 2
    rng = np.random.default_rng(11)
    a = rng.standard_normal((n, n))
    xact = rng.standard_normal((n, nrhs))
    b = a @ xact
    lu, ipiv, info = gpu.getrf(a)
    assert info == 0
    x0 = xact * (1 + 1e-6 * rng.standard_normal((n, nrhs)))
    x, ferr, berr, info = gpu.gerfs(a, lu, ipiv, b, x0, "N")
    assert info == 0
    r1, r2 = ck.dget07(a, b, x, xact, ferr, berr, "N")
    assert r1 < THRESH and r2 < THRESH, (r1, r2)
    assert np.all(berr < 10 * ck.EPS64 * (n + 1))
