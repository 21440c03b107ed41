"""Look-ahead schedule of the FP32 factorization (block column k+1 factored
on a second stream while the trailing update of block column k runs, its
row interchanges logged and replayed on the other columns afterwards).

The schedule changes when work runs, not what is computed: every element
sees the same updates in the same order as in the one-stream loop
(SRC/dgetrf.f:174-219).  So LU, IPIV and INFO are bitwise identical with
the look-ahead on and off, in every arithmetic mode, and bitwise identical
to the oracle in exact mode.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _rand(m, n, seed):
    return oracle.random_matrix(m, n, seed, idist=3, dtype=np.float32)[0]


class _opts:
    """Sets library options for a block and restores them after."""

    def __init__(self, g, **kv):
        self.g, self.kv, self.old = g, kv, {}

    def __enter__(self):
        for k, v in self.kv.items():
            self.old[k] = self.g.set_option(k, v)

    def __exit__(self, *a):
        for k, v in self.old.items():
            self.g.set_option(k, v)


@pytest.mark.parametrize("m,n,nb", [(700, 700, 64), (1000, 1000, 96), (900, 400, 64), (400, 900, 64),
                                    (520, 520, 256), (2048, 2048, 256)])
def test_lookahead_exact_bitwise_vs_oracle(gpu, exact_mode, m, n, nb):
    a = _rand(m, n, 7 + m + n)
    lu_r, ip_r, info_r = oracle.getrf(a)
    with _opts(gpu, nb32=nb, lookahead=1):
        lu_g, ip_g, info_g = gpu.getrf(a)
    assert info_g == info_r
    np.testing.assert_array_equal(ip_g, ip_r)
    assert lu_g.tobytes(order="F") == lu_r.tobytes(order="F"), "LU not bitwise identical"


@pytest.mark.parametrize("mode", [1, 0])            # sgetrf on FP32 CUDA cores / on BF16x3 tensor cores
@pytest.mark.parametrize("m,n,nb", [(1536, 1536, 256), (1300, 1100, 128), (3000, 3000, 256), (2500, 2500, 384)])
def test_lookahead_on_off_identical(gpu, mode, m, n, nb):
    a = _rand(m, n, 3 + m)
    with _opts(gpu, nb32=nb, sgetrf=mode, lookahead=0):
        lu0, ip0, info0 = gpu.getrf(a)
    with _opts(gpu, nb32=nb, sgetrf=mode, lookahead=1):
        lu1, ip1, info1 = gpu.getrf(a)
    assert info0 == info1
    np.testing.assert_array_equal(ip0, ip1)
    assert lu0.tobytes(order="F") == lu1.tobytes(order="F")


def test_lookahead_singular_info(gpu, exact_mode):
    a = _rand(800, 800, 19)
    a[:, 333] = 0.0                      # first zero pivot in the second block column
    lu_r, ip_r, info_r = oracle.getrf(a)
    with _opts(gpu, nb32=256, lookahead=1):
        lu_g, ip_g, info_g = gpu.getrf(a)
    assert info_r == 334 and info_g == info_r
    np.testing.assert_array_equal(ip_g, ip_r)
    assert lu_g.tobytes(order="F") == lu_r.tobytes(order="F")


def test_lookahead_dsgesv_identical(gpu):
    """DSGESV uses the running row permutation the logged interchanges
    update: its solution and ITER do not depend on the schedule."""
    n = 1800
    a, _, _, _ = oracle.config_dsgesv_matrix(n, 1e4, 5)
    b = a @ np.random.default_rng(5).standard_normal((n, 2))
    with _opts(gpu, nb32=256, lookahead=0):
        r0 = gpu.dsgesv(a, b)
    with _opts(gpu, nb32=256, lookahead=1):
        r1 = gpu.dsgesv(a, b)
    x0, it0, info0 = r0[2], r0[3], r0[4]
    x1, it1, info1 = r1[2], r1[3], r1[4]
    assert info0 == info1 == 0 and it0 == it1 and it0 > 0
    assert x0.tobytes() == x1.tobytes()


# grid-wide leaf / register cluster leaf / shared-memory cluster leaf (barrier exchange / pushed exchange)
@pytest.mark.parametrize("cluster_panel", [0, 1, 2, 3])
@pytest.mark.parametrize("m,n,nb", [(700, 700, 64), (1500, 1500, 256), (2100, 900, 128), (16384, 200, 64),
                                    (9000, 300, 256), (40, 37, 16)])
def test_panel_variants_exact_bitwise(gpu, exact_mode, cluster_panel, m, n, nb):
    """Every FP32 leaf kernel applies the DGETRF2 pivot and update rules in
    the reference order (SRC/dgetrf2.f:170-265): LU, IPIV and INFO match the
    oracle bit for bit whichever of them factors the leaves."""
    a = _rand(m, n, 41 + m + n)
    lu_r, ip_r, info_r = oracle.getrf(a)
    with _opts(gpu, nb32=nb, cluster_panel=cluster_panel):
        lu_g, ip_g, info_g = gpu.getrf(a)
    assert info_g == info_r
    np.testing.assert_array_equal(ip_g, ip_r)
    assert lu_g.tobytes(order="F") == lu_r.tobytes(order="F")


@pytest.mark.parametrize("cluster_panel", [1, 2, 3])
@pytest.mark.parametrize("m,n,nb", [(30000, 256, 256), (9000, 300, 256), (1500, 1500, 256)])
def test_panel_variants_default_mode_identical(gpu, cluster_panel, m, n, nb):
    """In the default (fused multiply-add) mode every leaf kernel still gives
    each element its updates in increasing k, one FMA each (the cluster
    leaves defer them in groups of four and apply the group in order), so
    SGETRF on the FP32 CUDA cores is bitwise the same whichever kernel
    factors the leaves."""
    a = _rand(m, n, 7 + m + n)
    with _opts(gpu, nb32=nb, sgetrf=1, cluster_panel=0):
        lu0, ip0, info0 = gpu.getrf(a)
    with _opts(gpu, nb32=nb, sgetrf=1, cluster_panel=cluster_panel):
        lu1, ip1, info1 = gpu.getrf(a)
    assert info0 == info1
    np.testing.assert_array_equal(ip0, ip1)
    assert lu0.tobytes(order="F") == lu1.tobytes(order="F")
