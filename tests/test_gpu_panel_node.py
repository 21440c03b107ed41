"""Fused node of the panel recursion (U12 = L11^{-1} A12 and A22 -= A21 U12
in one launch, SRC/dgetrf2.f:240-247) against the two separate launches.

The fused kernel does the solve in the order of the separate TRSM kernel
and folds k in increasing order into A22 as the separate update does, so
LU, IPIV and INFO are bitwise identical with the fusion on and off, in every
arithmetic mode; in exact mode they are bitwise those of the oracle.

The node shapes depend on the leaf width: tall FP32 panels (m about 30000)
get 24-column cluster leaves (nodes 24+24, 48+16, 64+64), m about 20000
32-column leaves (32+32, 64+64), shorter ones 64-column leaves (64+64);
FP64 with NB = 96 or 128 gets nodes 48+48 and 64+64.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _rand(m, n, seed, dtype):
    return oracle.random_matrix(m, n, seed, idist=3, dtype=dtype)[0]


class _opts:
    def __init__(self, g, **kv):
        self.g, self.kv, self.old = g, kv, {}

    def __enter__(self):
        for k, v in self.kv.items():
            self.old[k] = self.g.set_option(k, v)

    def __exit__(self, *a):
        for k, v in self.old.items():
            self.g.set_option(k, v)


def _same(r0, r1):
    lu0, ip0, info0 = r0
    lu1, ip1, info1 = r1
    assert info0 == info1
    np.testing.assert_array_equal(ip0, ip1)
    assert lu0.tobytes(order="F") == lu1.tobytes(order="F"), "LU not bitwise identical"


FP32_SHAPES = [(30000, 256, 256), (30001, 200, 256), (20000, 192, 128), (4100, 300, 256), (1000, 1000, 128)]


@pytest.mark.parametrize("m,n,nb", FP32_SHAPES)
@pytest.mark.parametrize("mode", [1, 0])            # sgetrf on FP32 CUDA cores / on BF16x3 tensor cores
@pytest.mark.parametrize("la", [0, 1])
def test_fp32_fused_node_matches_separate_launches(gpu, m, n, nb, mode, la):
    a = _rand(m, n, m + 3 * n, np.float32)
    with _opts(gpu, nb32=nb, sgetrf=mode, lookahead=la, panel_fuse=0):
        r0 = gpu.getrf(a)
    with _opts(gpu, nb32=nb, sgetrf=mode, lookahead=la, panel_fuse=1):
        r1 = gpu.getrf(a)
    _same(r0, r1)


@pytest.mark.parametrize("m,n,nb", [(30000, 256, 256), (20000, 130, 128), (900, 700, 128)])
def test_fp32_fused_node_exact_bitwise_vs_oracle(gpu, exact_mode, m, n, nb):
    a = _rand(m, n, 11 + m + n, np.float32)
    ref = oracle.getrf(a)
    with _opts(gpu, nb32=nb, panel_fuse=1):
        got = gpu.getrf(a)
    _same(ref, got)


@pytest.mark.parametrize("m,n,nb", [(3000, 3000, 128), (2500, 700, 96), (700, 2500, 128), (1000, 1000, 96)])
def test_fp64_fused_node_matches_separate_launches(gpu, m, n, nb):
    a = _rand(m, n, 5 + m, np.float64)
    with _opts(gpu, nb64=nb, panel_fuse=0):
        r0 = gpu.getrf(a)
    with _opts(gpu, nb64=nb, panel_fuse=1):
        r1 = gpu.getrf(a)
    _same(r0, r1)


@pytest.mark.parametrize("m,n,nb", [(1500, 1500, 128), (1200, 500, 96)])
def test_fp64_fused_node_exact_bitwise_vs_oracle(gpu, exact_mode, m, n, nb):
    a = _rand(m, n, 29 + m, np.float64)
    ref = oracle.getrf(a)
    with _opts(gpu, nb64=nb, panel_fuse=1):
        got = gpu.getrf(a)
    _same(ref, got)


def test_fused_node_singular_column(gpu, exact_mode):
    """A zero column inside a fused node's right half: INFO and the factors
    as the oracle's (the node's solve and update see the zero pivot's
    column like the separate launches do)."""
    a = _rand(20000, 128, 41, np.float32)
    a[:, 70] = 0.0
    ref = oracle.getrf(a)
    with _opts(gpu, nb32=128, panel_fuse=1):
        got = gpu.getrf(a)
    assert ref[2] == 71
    _same(ref, got)


def test_fused_node_dsgesv_identical(gpu):
    """DSGESV's FP32 factorization (BF16x3 mode, look-ahead) with the fusion
    on and off: the same solution and iteration count."""
    n = 3000
    a, _, _, _ = oracle.config_dsgesv_matrix(n, 1e4, 8)
    b = a @ np.random.default_rng(8).standard_normal((n, 2))
    outs = []
    for fuse in (0, 1):
        with _opts(gpu, panel_fuse=fuse):
            outs.append(gpu.dsgesv(a, b))
    x0, x1 = outs[0][2], outs[1][2]
    assert outs[0][3] == outs[1][3]            # ITER
    assert x0.tobytes() == x1.tobytes()
