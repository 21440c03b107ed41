"""Fixture for the full-size FP64 DGESV configuration: n = 16384, nrhs = 16,
A iid U[-1,1] (DLARNV idist 2) and B iid N(0,1) (idist 3) drawn next from
the stream of scalar seed 1 (ISEED = {0, 0, 0, 3}).

The oracle (the C restatement of SRC/dgetrf.f, SRC/dgetrf2.f, SRC/dgetrs.f
with the reference BLAS loops, NB = 64, column-parallel over the host cores)
factors the matrix once; too slow to run inside a test, so the figures the
GPU test compares against are cached here:

  * sha256 of A and B as generated (the test regenerates them and checks);
  * IPIV and the relative pivot margin of every column;
  * the column sums of the LU factors and a strided sample LU[::128, ::128];
  * the oracle's X sampled every 16th row, its scaled residual
    ||b - A x||_inf / (||A||_inf ||x||_inf n eps) and its DGET02 ratio
    ||b - A x||_1 / (||A||_1 ||x||_1 eps), per right-hand side.

    python tests/golden/make_config2.py      (a few minutes on 8 cores)
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

OUT = os.path.join(HERE, "dgesv_n16384_nrhs16_seed1.npz")
N, NRHS, SEED, STRIDE, XSTRIDE = 16384, 16, 1, 128, 16
EPS = 2.0 ** -53


def main():
    t0 = time.time()
    a, b = oracle.config_dgesv_fp64(N, NRHS, SEED)
    sha_a = hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()
    sha_b = hashlib.sha256(np.asfortranarray(b).tobytes(order="F")).hexdigest()
    lu, ipiv, info, margin = oracle.getrf(a, nb=64, margins=True)
    assert info == 0, info
    t_f = time.time() - t0
    x, info = oracle.getrs(lu, ipiv, b)
    assert info == 0
    r = b - a @ x
    anrm_inf = np.abs(a).sum(axis=1).max()
    anrm_1 = np.abs(a).sum(axis=0).max()
    scaled = np.array([np.abs(r[:, j]).max() / (anrm_inf * np.abs(x[:, j]).max() * N * EPS) for j in range(NRHS)])
    dget02 = np.array([np.abs(r[:, j]).sum() / (anrm_1 * np.abs(x[:, j]).sum() * EPS) for j in range(NRHS)])
    np.savez_compressed(
        OUT, n=N, nrhs=NRHS, seed=SEED, sha_a=sha_a, sha_b=sha_b, ipiv=ipiv.astype(np.int32),
        margin=margin, colsum=lu.sum(axis=0), lu_sample=np.ascontiguousarray(lu[::STRIDE, ::STRIDE]),
        stride=STRIDE, x_sample=np.ascontiguousarray(x[::XSTRIDE]), xstride=XSTRIDE, scaled_residual=scaled,
        dget02=dget02)
    print(f"factor {t_f:.1f} s, total {time.time() - t0:.1f} s; scaled residual max {scaled.max():.3e}, "
          f"DGET02 max {dget02.max():.3e}, min margin {margin.min():.3e} -> {OUT}")


if __name__ == "__main__":
    main()
