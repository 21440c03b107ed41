"""DGETRI on the GPU (SRC/dgetri.f) against the oracle's restatement.

Exact mode: the inverse bitwise equal to the oracle's DGETRI for block sizes
1 (unblocked), 3, 20, 64 (the reference's ILAENV value) and a block size at
least N, over the DCHKGE matrix types; INFO = the first zero pivot of U.
Default mode: DCHKGE test 2 (TESTING/LIN/dchkge.f:383-420, DGET03 below
THRESH)."""
import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu
THRESH = 30.0


class _nb:
    def __init__(self, g, nb):
        self.g, self.nb = g, nb

    def __enter__(self):
        self.old = self.g.set_option("nb64", self.nb)

    def __exit__(self, *a):
        self.g.set_option("nb64", self.old)


@pytest.mark.parametrize("nb", [1, 3, 20, 64, 512])
@pytest.mark.parametrize("n,imat", [(1, 1), (2, 2), (7, 3), (65, 4), (130, 1), (300, 9), (300, 6)])
def test_getri_exact_bitwise(gpu, exact_mode, nb, n, imat):
    a, izero = oracle.ge_test_matrix(n, n, imat, 23 + n + imat)
    lu, ipiv, info = oracle.getrf(a)
    ref, rinfo, rw = oracle.getri(lu, ipiv, nb=nb)
    with _nb(gpu, nb):
        got, ginfo, gw = gpu.getri(lu, ipiv)
    assert ginfo == rinfo
    if rinfo == 0:
        assert got.tobytes(order="F") == np.asfortranarray(ref).tobytes(order="F")
        assert gw == rw


def test_getri_small_workspace_exact(gpu, exact_mode):
    """LWORK below N*NB: the block size shrinks to LWORK/N as in the reference."""
    n = 130
    a = oracle.random_matrix(n, n, 5, idist=3)[0]
    lu, ipiv, _ = oracle.getrf(a)
    ref, _, rw = oracle.getri(lu, ipiv, nb=64, lwork=n * 5)
    with _nb(gpu, 64):
        got, info, gw = gpu.getri(lu, ipiv, lwork=n * 5)
    assert info == 0 and gw == rw
    assert got.tobytes(order="F") == np.asfortranarray(ref).tobytes(order="F")


@pytest.mark.parametrize("imat", range(1, 12))
def test_getri_dchkge_ratio(gpu, imat):
    for n in (3, 10, 50, 200, 600):
        if 5 <= imat <= 7 and n < imat - 4:
            continue
        a, izero = oracle.ge_test_matrix(n, n, imat, 1988 + 11 * n)
        lu, ipiv, info = gpu.getrf(a)
        ainv, info, _ = gpu.getri(lu, ipiv)
        if izero:
            assert info > 0
            continue
        assert info == 0
        assert ck.dget03(a, ainv)[0] < THRESH, (n, imat)


def test_getri_device_api_matches_host_abi(gpu):
    import torch
    n = 257
    a = oracle.random_matrix(n, n, 9, idist=3)[0]
    lu, ipiv, _ = oracle.getrf(a)
    host, info, _ = gpu.getri(lu, ipiv)
    A = gpu.to_colmajor(lu)
    ip = torch.from_numpy(np.ascontiguousarray(ipiv, dtype=np.int32)).cuda()
    import ctypes
    inf = ctypes.c_int(0)
    ld, pa = gpu._colmajor_view(A)
    rc = gpu.lib().gb300_dgetri_dev(n, ctypes.c_void_p(pa), ld, ctypes.c_void_p(ip.data_ptr()), ctypes.byref(inf),
                                    gpu._stream_ptr(None))
    torch.cuda.synchronize()
    assert rc == 0 and inf.value == 0 == info
    assert A.cpu().numpy().tobytes(order="F") == np.asfortranarray(host).tobytes(order="F")
