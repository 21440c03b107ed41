"""Batched uneven-size DGESV / SGESV (one persistent launch) against the
oracle's DGESV / SGESV applied to each system (SRC/dgesv.f).

* exact mode: LU, IPIV, X and INFO bitwise equal to the oracle per system;
* default mode: IPIV equal, scaled residual within 2x the oracle's;
* a singular member reports its INFO without disturbing the others;
* the launch sequence captured in a CUDA graph and replayed gives the same
  results as the eager call.
"""
import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu


def make_batch(count, seed, nmin=8, nmax=512, dtype=np.float64):
    """n uniform in [nmin, nmax], nrhs in {1, 2, 4}, entries N(0,1) with n*I
    added to every other system (the batched configuration's construction)."""
    rng = np.random.default_rng(seed)
    ns = list(rng.integers(nmin, nmax + 1, count))
    ns[:6] = [1, 2, 63, 64, 65, nmax][: min(6, count)]
    As, Bs = [], []
    for i, n in enumerate(ns):
        a = oracle.random_matrix(int(n), int(n), seed * 1000 + i, idist=3)[0]
        if i % 2 == 0:
            a = a + n * np.eye(n)
        nrhs = int(rng.choice([1, 2, 4]))
        b = oracle.random_matrix(int(n), nrhs, seed * 1000 + 500 + i, idist=3)[0]
        As.append(a.astype(dtype))
        Bs.append(b.astype(dtype))
    return As, Bs


@pytest.mark.parametrize("dt", ["d", "s"])
def test_batched_exact_bitwise(gpu, exact_mode, dt):
    import torch
    dtype = np.float64 if dt == "d" else np.float32
    As, Bs = make_batch(24, 7, dtype=dtype)
    lus, ips, xs, info = gpu.gesv_vbatched(As, Bs, torch.float64 if dt == "d" else torch.float32)
    for i, (a, b) in enumerate(zip(As, Bs)):
        lu_r, ip_r, x_r, info_r = oracle.gesv(a, b)
        assert info[i] == info_r
        np.testing.assert_array_equal(ips[i], ip_r)
        assert lus[i].tobytes() == np.asfortranarray(lu_r).tobytes(), f"system {i} n={a.shape[0]}"
        assert xs[i].tobytes() == np.asfortranarray(x_r).tobytes(), f"system {i} n={a.shape[0]}"


def test_batched_default_parity(gpu):
    As, Bs = make_batch(40, 11)
    lus, ips, xs, info = gpu.gesv_vbatched(As, Bs)
    for i, (a, b) in enumerate(zip(As, Bs)):
        lu_r, ip_r, x_r, info_r = oracle.gesv(a, b, )
        assert info[i] == info_r == 0
        np.testing.assert_array_equal(ips[i], ip_r)
        assert ck.scaled_residual(a, xs[i], b) <= max(2 * ck.scaled_residual(a, x_r, b), 1e-3)


def test_batched_singular_member(gpu):
    As, Bs = make_batch(8, 13, nmax=100)
    As[3] = As[3].copy()
    As[3][:, 4] = 0.0
    lus, ips, xs, info = gpu.gesv_vbatched(As, Bs)
    _, _, _, info_r = oracle.gesv(As[3], Bs[3])
    assert info[3] == info_r == 5
    np.testing.assert_array_equal(xs[3], Bs[3])                 # solve skipped, B unchanged
    for i in range(8):
        if i != 3:
            assert info[i] == 0 and ck.dget02(As[i], xs[i], Bs[i]) < 30.0


def test_batched_graph_capture(gpu):
    import torch
    As, Bs = make_batch(16, 17)
    eager = gpu.VBatch(As, Bs)
    eager.launch()
    torch.cuda.synchronize()
    ref = eager.results()
    vb = gpu.VBatch(As, Bs)
    a0, b0 = vb.A.clone(), vb.B.clone()  # the inputs, before any launch factors them in place
    vb.launch()                          # warm-up outside the capture (sets kernel attributes)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        vb.A.copy_(a0)
        vb.B.copy_(b0)
        g.capture_begin()
        vb.launch(stream=s)
        g.capture_end()
    for _ in range(2):
        vb.A.copy_(a0)
        vb.B.copy_(b0)
        g.replay()
        torch.cuda.synchronize()
        got = vb.results()
        for i in range(len(As)):
            assert np.array_equal(got[1][i], ref[1][i])
            assert np.array_equal(got[2][i], ref[2][i])


@pytest.mark.parametrize("dt", ["d", "s"])
@pytest.mark.parametrize("nb", [1, 3, 5, 8, 13, 32])
def test_batched_exact_bitwise_panel_widths(gpu, exact_mode, dt, nb):
    """Panel widths that are not multiples of the four columns whose
    updates the panel defers (and the single-column panel): the factors and
    solutions stay bitwise the oracle's."""
    import torch
    dtype = np.float64 if dt == "d" else np.float32
    code = 0 if dt == "d" else 1
    old = gpu.vbatched_nb(code)
    gpu.set_vbatched_nb(code, [nb] * 8)
    try:
        As, Bs = make_batch(10, 29 + nb, nmax=300, dtype=dtype)
        lus, ips, xs, info = gpu.gesv_vbatched(As, Bs, torch.float64 if dt == "d" else torch.float32)
    finally:
        gpu.set_vbatched_nb(code, old)
    for i, (a, b) in enumerate(zip(As, Bs)):
        lu_r, ip_r, x_r, info_r = oracle.gesv(a, b)
        assert info[i] == info_r
        np.testing.assert_array_equal(ips[i], ip_r)
        assert lus[i].tobytes() == np.asfortranarray(lu_r).tobytes(), f"system {i} n={a.shape[0]}"
        assert xs[i].tobytes() == np.asfortranarray(x_r).tobytes(), f"system {i} n={a.shape[0]}"
