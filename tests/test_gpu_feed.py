"""Host-pointer DSGESV with A copied in column chunks beside the FP32
factorization (option "feed") against the copy-everything-first path
(feed = 0).

The factorization takes a chunk in when it has landed (or, with
"feed_lazy", only when the next block columns need it); a chunk taken in
after block columns 0..k-1 were factored first gets their interchanges and
then, block column by block column in order, their U rows and trailing
updates -- the operations the right-looking loop (SRC/dgetrf.f:174-219)
applies to every column, in the same order.  The conversion of a chunk
(DLAG2S, SRC/dlag2s.f) and its DLANGE row sums (SRC/dlange.f:173-189) use
the column split of the one-pass kernel, or one running sum per row in
exact mode.  So X, ITER, INFO, IPIV and the returned A are bitwise the same
with and without the overlap, in every arithmetic mode and for every exit
of SRC/dsgesv.f (converged, -2 overflow, -3 singular FP32 factor).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


class _opts:
    def __init__(self, g, **kv):
        self.g, self.kv, self.old = g, kv, {}

    def __enter__(self):
        for k, v in self.kv.items():
            self.old[k] = self.g.set_option(k, v)

    def __exit__(self, *a):
        for k, v in self.old.items():
            self.g.set_option(k, v)


def _system(n, nrhs, seed, kappa=1e4):
    a, _, _, _ = oracle.config_dsgesv_matrix(n, kappa, seed)
    b = a @ np.random.default_rng(seed).standard_normal((n, nrhs))
    return a, b


def _same(r0, r1):
    a0, ip0, x0, it0, info0 = r0
    a1, ip1, x1, it1, info1 = r1
    assert (it0, info0) == (it1, info1)
    np.testing.assert_array_equal(ip0, ip1)
    assert x0.tobytes() == x1.tobytes(), "X not bitwise identical"
    assert a0.tobytes() == a1.tobytes(), "returned A not bitwise identical"


def _both(gpu, a, b, **kv):
    with _opts(gpu, feed=0, **kv):
        r0 = gpu.dsgesv(a, b)
    with _opts(gpu, feed=1, **kv):
        r1 = gpu.dsgesv(a, b)
    return r0, r1


@pytest.mark.parametrize("n,nrhs", [(600, 1), (3000, 1), (5000, 3), (8192, 2)])
@pytest.mark.parametrize("lazy", [0, 1, 2])
@pytest.mark.parametrize("mixed", [0, 1])          # BF16x3 tensor cores / FP32 CUDA cores
def test_fed_dsgesv_matches_whole_copy(gpu, n, nrhs, lazy, mixed):
    a, b = _system(n, nrhs, 3 + n)
    r0, r1 = _both(gpu, a, b, feed_lazy=lazy, mixed=mixed)
    _same(r0, r1)
    assert r1[3] >= 0 and r1[4] == 0


@pytest.mark.parametrize("catchup", [0, 1, 3, 8])
@pytest.mark.parametrize("mixed", [0, 1])
def test_fed_dsgesv_spread_catchup(gpu, catchup, mixed):
    """A chunk taken in at every step (feed_lazy 2) while the ones before
    are still catching up a few block columns per step (catchup; 0: all at
    once): the pending columns take every later interchange with the rest
    of the matrix and join when current -- same bits."""
    n = 9000                                      # 16 chunks of 563 columns, 36 block columns
    a, b = _system(n, 1, 7)
    r0, r1 = _both(gpu, a, b, feed_lazy=2, feed_catchup=catchup, mixed=mixed)
    _same(r0, r1)


@pytest.mark.parametrize("n", [2500, 4500])
@pytest.mark.parametrize("lazy", [0, 1, 2])
def test_fed_dsgesv_exact_matches_whole_copy_and_oracle(gpu, exact_mode, n, lazy):
    """Exact mode with the FP32 CUDA-core factorization (the SGETRF
    arithmetic): 2048-column chunks continue one running row sum; the result
    is also the oracle's, bit for bit."""
    a, b = _system(n, 2, 17 + n)
    r0, r1 = _both(gpu, a, b, feed_lazy=lazy, mixed=1)
    _same(r0, r1)
    _, ip_r, x_r, it_r, info_r = oracle.dsgesv(a, b)
    assert (r1[3], r1[4]) == (it_r, info_r)
    np.testing.assert_array_equal(r1[1], ip_r)
    assert r1[2].tobytes() == np.asfortranarray(x_r).tobytes()


@pytest.mark.parametrize("col", [5, 2999])
def test_fed_dsgesv_overflow_in_a_chunk(gpu, col):
    """An entry beyond FP32 range in the first or the last chunk: DLAG2S
    fails, ITER = -2, and the FP64 factorization solves (SRC/dsgesv.f:
    274-281); the late case stops the fed factorization part-way."""
    n = 3000
    a, b = _system(n, 1, 29)             # B itself stays in FP32 range
    a[7, col] = 1e39
    for lazy in (0, 1):
        r0, r1 = _both(gpu, a, b, feed_lazy=lazy)
        _same(r0, r1)
        assert r1[3] == -2


def test_fed_dsgesv_singular_fp32_factor(gpu):
    """A column that underflows to zero in FP32 (but not in FP64) makes
    SGETRF report INFO > 0: ITER = -3, the FP64 solve (SRC/dsgesv.f:
    297-301)."""
    n = 3000
    a, b = _system(n, 1, 31)
    a[:, 2500] *= 1e-50
    b = a @ np.ones((n, 1))
    r0, r1 = _both(gpu, a, b)
    _same(r0, r1)
    assert r1[3] == -3


def test_fed_dsgesv_repeated_calls(gpu):
    """Consecutive calls reuse the workspace, the streams and the flag
    words: each call still sees only its own chunks."""
    n = 4096
    outs = []
    for seed in (41, 42, 41):
        a, b = _system(n, 1, seed)
        with _opts(gpu, feed=1):
            outs.append(gpu.dsgesv(a, b))
    assert outs[0][2].tobytes() == outs[2][2].tobytes()
    assert outs[0][2].tobytes() != outs[1][2].tobytes()
