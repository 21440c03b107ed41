// DGERFS and DGECON on the GPU.
//
// DGERFS (SRC/dgerfs.f:186-424): iterative refinement of the
// solutions X of op(A) X = B with the LU factors AF/IPIV, the componentwise
// backward error BERR, and the forward error bound FERR from the DLACN2
// estimate of || |inv(op(A))| (|R| + NZ*EPS*(|op(A)||X| + |B|)) ||.
//
// All vectors stay in device memory.  The host only reads, per pass, the
// BERR values (to apply the reference's stopping test column by column)
// and, per estimator step, each column's KASE (to group the columns that
// need a solve with op(A) and with op(A)^T into one multi-right-hand-side
// DGETRS each).  A column's arithmetic does not depend on which other
// columns share a pass, so X, FERR and BERR of each column are those of the
// reference's one-column-at-a-time loop; in exact mode they are bitwise the
// reference's.
//
// DGECON (SRC/dgecon.f:166-252): the same DLACN2 steps on one device vector,
// each product with inv(A) or inv(A)^T done as two DLATRS solves
// (SRC/dlatrs.f) whose CNORM vectors are computed once; the host reads the
// estimator state and each DLATRS plan (DTRSV or the careful solve).
#include "driver.h"
#include "prof.h"
#include "condest_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace gb {

namespace {

unsigned blocks256(size_t n) { return (unsigned)((n + 255) / 256); }

// Splits a column set into launch lists of at most kRfsMaxList entries.
std::vector<ColList> make_lists(const std::vector<int>& cols) {
  std::vector<ColList> out;
  for (size_t b = 0; b < cols.size(); b += kRfsMaxList) {
    ColList l{};
    l.n = (int)std::min<size_t>(kRfsMaxList, cols.size() - b);
    for (int t = 0; t < l.n; ++t) l.c[t] = cols[b + t];
    out.push_back(l);
  }
  return out;
}

// R(:, c) = B(:, c) - op(A) X(:, c) and W(:, c) = |B(:, c)| + |op(A)||X(:, c)|
// for the listed columns.
int residual_bound(bool notran, int n, const double* A, int lda, const double* B, int ldb, const double* X, int ldx,
                   double* R, double* W, int ldr, const ColList& cols, cudaStream_t s) {
  prof_begin(kProfResidual, s);
  if (options().exact) {
    dim3 g((unsigned)((n + 127) / 128), (unsigned)cols.n);
    if (notran) GB_LAUNCH(rfs_resid_exact_kernel<false><<<g, 128, 0, s>>>(A, lda, B, ldb, X, ldx, R, W, ldr, n, cols));
    else GB_LAUNCH(rfs_resid_exact_kernel<true><<<g, 128, 0, s>>>(A, lda, B, ldb, X, ldx, R, W, ldr, n, cols));
  } else if (notran) {
    // column chunks depend on n only (never on how many columns share the
    // pass), so each column's sums are the same alone or in a batch
    int nsplit = std::max(1, std::min(16, n / 256));
    int chunk = ((n + nsplit - 1) / nsplit + 31) / 32 * 32;
    nsplit = (n + chunk - 1) / chunk;
    DevScratch part(sizeof(double) * (size_t)nsplit * kRfsRq * 2 * n, s);
    if (!part.p) return (int)cudaErrorMemoryAllocation;
    const unsigned rows = (unsigned)((n + kRfsRows - 1) / kRfsRows);
    for (int t0 = 0; t0 < cols.n; t0 += kRfsRq) {
      ColList sub{};
      sub.n = std::min(kRfsRq, cols.n - t0);
      for (int t = 0; t < sub.n; ++t) sub.c[t] = cols.c[t0 + t];
      dim3 g(rows, nsplit, 1);
      GB_LAUNCH(rfs_resid_partial_n_kernel<<<g, kRfsRows, 0, s>>>(A, lda, X, ldx, n, chunk, sub, part.as<double>()));
      GB_LAUNCH(rfs_resid_fold_kernel<<<blocks256((size_t)n * sub.n), 256, 0, s>>>(part.as<double>(), nsplit, B, ldb,
                                                                                     R, W, ldr, n, sub));
    }
  } else {
    dim3 g((unsigned)((n + 7) / 8), (unsigned)((cols.n + kRfsRq - 1) / kRfsRq));
    GB_LAUNCH(rfs_resid_t_kernel<<<g, 256, 0, s>>>(A, lda, B, ldb, X, ldx, R, W, ldr, n, cols));
  }
  prof_end(kProfResidual, s, 4.0 * n * (double)n * cols.n, 8.0 * ((double)n * n + 4.0 * n * cols.n));
  return (int)cudaGetLastError();
}

// D(:, 0..k-1) = Src(:, cols) [times Wpre(:, cols)], one DGETRS with op = `t`
// on D, then Dst(:, cols) = D [times Wpost(:, cols)], or Dst(:, cols) += D.
int solve_listed(char t, int n, const double* AF, int ldaf, const int* ipiv, const int* perm, const double* Src,
                 int lds, const double* Wpre, double* Dst, int ldd, const double* Wpost, int ldw, bool add,
                 const std::vector<int>& cols, double* D, cudaStream_t s) {
  const int k = (int)cols.size();
  if (k == 0) return 0;
  std::vector<ColList> lists = make_lists(cols);
  int base = 0;
  for (const ColList& l : lists) {
    GB_LAUNCH(rfs_gather_kernel<<<blocks256((size_t)n * l.n), 256, 0, s>>>(Src, lds, Wpre, ldw, D, n, n, l, base));
    base += l.n;
  }
  int rc = getrs_dev<double>(t, n, k, AF, ldaf, ipiv, perm, D, n, s);
  if (rc) return rc;
  base = 0;
  for (const ColList& l : lists) {
    GB_LAUNCH(rfs_scatter_kernel<<<blocks256((size_t)n * l.n), 256, 0, s>>>(D, n, Wpost, ldw, Dst, ldd, n, l, base,
                                                                            add ? 1 : 0));
    base += l.n;
  }
  return (int)cudaGetLastError();
}

// One DLATRS call on the device vector x: the triangle of A selected by
// `upper`, op = N (notran) or T, unit or non-unit diagonal.  CNORM is
// computed unless normin_y; the plan (and SCALE) goes to *plan.
int latrs_dev(bool upper, bool notran, bool unit, int n, const double* A, int lda, double* x, double* cnorm,
              bool normin_y, LatrsPlan* plan, cudaStream_t s) {
  const bool ex = options().exact;
  const int nounit = unit ? 0 : 1;
  if (!normin_y) {
    if (ex) GB_LAUNCH(latrs_cnorm_kernel<true><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(upper, n, A, lda, cnorm));
    else GB_LAUNCH(latrs_cnorm_kernel<false><<<(unsigned)((n + 7) / 8), 256, 0, s>>>(upper, n, A, lda, cnorm));
  }
  GB_LAUNCH(latrs_plan_kernel<<<1, 1, 0, s>>>(upper, notran, nounit, n, A, lda, x, cnorm, plan));
  LatrsPlan hp;
  GB_CUDA_TRY(cudaMemcpyAsync(&hp, plan, sizeof(hp), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  if (hp.mode == kLatrsCareful) {
    GB_LAUNCH(latrs_careful_kernel<<<1, 1, 0, s>>>(upper, notran, nounit, n, A, lda, x, cnorm, plan));
    return (int)cudaGetLastError();
  }
  // DTRSV (dlatrs.f:499-503, or :395 when even TMAX overflows)
  return dtrsv_dev(upper, !notran, unit, n, A, lda, x, s);
}

}  // namespace

int dgerfs_dev(char trans, int n, int nrhs, const double* A, int lda, const double* AF, int ldaf, const int* ipiv,
               const double* B, int ldb, double* X, int ldx, double* ferr, double* berr, cudaStream_t s) {
  if (nrhs <= 0) return 0;
  if (n <= 0) {   // SRC/dgerfs.f:263-269
    GB_CUDA_TRY(cudaMemsetAsync(ferr, 0, sizeof(double) * nrhs, s));
    GB_CUDA_TRY(cudaMemsetAsync(berr, 0, sizeof(double) * nrhs, s));
    return 0;
  }
  const bool notran = (trans == 'N' || trans == 'n');
  const char tr = notran ? 'N' : 'T', trt = notran ? 'T' : 'N';
  const int itmax = 5;                                   // SRC/dgerfs.f:208
  const int nz = n + 1;
  const double eps = 1.1102230246251565e-16;             // DLAMCH('Epsilon')
  const double safmin = 2.2250738585072014e-308;         // DLAMCH('Safe minimum')
  const double safe1 = nz * safmin, safe2 = safe1 / eps;

  const size_t vec = (size_t)n * nrhs;
  DevScratch perm(sizeof(int) * (size_t)n, s), rw(sizeof(double) * vec * 5, s), ib(sizeof(int) * vec, s),
      stb(sizeof(LacnState) * (size_t)nrhs, s);
  if (!perm.p || !rw.p || !ib.p || !stb.p) return (int)cudaErrorMemoryAllocation;
  double* R = rw.as<double>();
  double* W = R + vec;
  double* D = W + vec;
  double* Xe = D + vec;
  double* V = Xe + vec;
  int* Isgn = ib.as<int>();
  LacnState* st = stb.as<LacnState>();
  int rc = ipiv_perm_dev(ipiv, 1, n, 1, 0, n, perm.as<int>(), s);
  if (rc) return rc;

  // ---- refinement (SRC/dgerfs.f:286-399)
  std::vector<int> active(nrhs), count(nrhs, 1);
  std::vector<double> lstres(nrhs, 3.0), hberr(nrhs);
  for (int j = 0; j < nrhs; ++j) active[j] = j;
  while (!active.empty()) {
    for (const ColList& l : make_lists(active)) {
      if ((rc = residual_bound(notran, n, A, lda, B, ldb, X, ldx, R, W, n, l, s))) return rc;
      GB_LAUNCH(rfs_berr_kernel<<<l.n, 256, 0, s>>>(R, W, n, n, safe1, safe2, l, berr));
    }
    GB_CUDA_TRY(cudaMemcpyAsync(hberr.data(), berr, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<int> again;
    for (int j : active) {
      if (hberr[j] > eps && 2.0 * hberr[j] <= lstres[j] && count[j] <= itmax) {
        again.push_back(j);
        lstres[j] = hberr[j];
        count[j] += 1;
      }
    }
    // X(:, j) += op(A)^{-1} R(:, j) for the columns that refine again
    if ((rc = solve_listed(tr, n, AF, ldaf, ipiv, perm.as<int>(), R, n, nullptr, X, ldx, nullptr, n, true, again, D,
                           s)))
      return rc;
    active.swap(again);
  }

  // ---- forward error bound (SRC/dgerfs.f:401-459)
  std::vector<int> all(nrhs);
  for (int j = 0; j < nrhs; ++j) all[j] = j;
  const double nzeps = (double)nz * eps;
  const bool ex = options().exact;
  GB_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(LacnState) * (size_t)nrhs, s));
  for (const ColList& l : make_lists(all)) {
    GB_LAUNCH(rfs_ferr_weights_kernel<<<blocks256((size_t)n * l.n), 256, 0, s>>>(R, W, n, n, nzeps, safe1, safe2, l));
    if (ex) GB_LAUNCH(lacn2_step_kernel<true><<<l.n, 256, 0, s>>>(n, Xe, n, V, Isgn, st, l));
    else GB_LAUNCH(lacn2_step_kernel<false><<<l.n, 256, 0, s>>>(n, Xe, n, V, Isgn, st, l));
  }
  std::vector<LacnState> hst(nrhs);
  for (;;) {
    GB_CUDA_TRY(cudaMemcpyAsync(hst.data(), st, sizeof(LacnState) * (size_t)nrhs, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<int> g1, g2;
    for (int j = 0; j < nrhs; ++j) {
      if (hst[j].kase == 1) g1.push_back(j);
      else if (hst[j].kase == 2) g2.push_back(j);
    }
    if (g1.empty() && g2.empty()) break;
    // KASE 1: x := diag(W) op(A)^{-T} x;  KASE 2: x := op(A)^{-1} diag(W) x
    if ((rc = solve_listed(trt, n, AF, ldaf, ipiv, perm.as<int>(), Xe, n, nullptr, Xe, n, W, n, false, g1, D, s)))
      return rc;
    if ((rc = solve_listed(tr, n, AF, ldaf, ipiv, perm.as<int>(), Xe, n, W, Xe, n, nullptr, n, false, g2, D, s)))
      return rc;
    std::vector<int> both(g1);
    both.insert(both.end(), g2.begin(), g2.end());
    for (const ColList& l : make_lists(both)) {
      if (ex) GB_LAUNCH(lacn2_step_kernel<true><<<l.n, 256, 0, s>>>(n, Xe, n, V, Isgn, st, l));
      else GB_LAUNCH(lacn2_step_kernel<false><<<l.n, 256, 0, s>>>(n, Xe, n, V, Isgn, st, l));
    }
  }
  for (const ColList& l : make_lists(all))
    GB_LAUNCH(rfs_ferr_finish_kernel<<<l.n, 256, 0, s>>>(X, ldx, n, st, l, ferr));
  return (int)cudaGetLastError();
}

int dgecon_dev(char norm, int n, const double* LU, int lda, double anorm, double* rcond, int* info,
               cudaStream_t s) {
  // SRC/dgecon.f:197-212 (argument errors are the caller's)
  const double hugeval = kOvfl;
  const bool onenrm = (norm == '1' || norm == 'O' || norm == 'o');
  *info = 0;
  *rcond = 0.0;
  if (n == 0) { *rcond = 1.0; return 0; }
  if (anorm == 0.0) return 0;
  if (anorm != anorm) { *rcond = anorm; *info = -5; return 0; }
  if (anorm > hugeval) { *info = -5; return 0; }
  DevScratch vb(sizeof(double) * 4 * (size_t)n, s), ib(sizeof(int) * (size_t)n + 256, s),
      sb(sizeof(LacnState) + 2 * sizeof(LatrsPlan) + 64, s);
  if (!vb.p || !ib.p || !sb.p) return (int)cudaErrorMemoryAllocation;
  double* x = vb.as<double>();
  double* v = x + n;
  double* cl = v + n;
  double* cu = cl + n;
  int* isgn = ib.as<int>();
  int* stop = isgn + n;
  LacnState* st = sb.as<LacnState>();
  LatrsPlan* plans = reinterpret_cast<LatrsPlan*>(sb.as<char>() + 64);   // [0] L, [1] U
  GB_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(LacnState), s));
  GB_CUDA_TRY(cudaMemsetAsync(stop, 0, sizeof(int), s));
  const bool ex = options().exact;
  ColList one{};
  one.n = 1;
  one.c[0] = 0;
  const int kase1 = onenrm ? 1 : 2;
  bool normin_y = false;
  int rc;
  for (int guard = 0; guard < 64; ++guard) {
    if (ex) GB_LAUNCH(lacn2_step_kernel<true><<<1, 256, 0, s>>>(n, x, n, v, isgn, st, one));
    else GB_LAUNCH(lacn2_step_kernel<false><<<1, 256, 0, s>>>(n, x, n, v, isgn, st, one));
    LacnState hs;
    GB_CUDA_TRY(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hs.kase == 0) {
      // RCOND = (1/AINVNM)/ANORM (dgecon.f:242-250)
      if (hs.est != 0.0) {
        *rcond = (1.0 / hs.est) / anorm;
      } else {
        *info = 1;
        return 0;
      }
      if (*rcond != *rcond || *rcond > hugeval) *info = 1;
      return 0;
    }
    if (hs.kase == kase1) {   // inv(L) then inv(U)
      if ((rc = latrs_dev(false, true, true, n, LU, lda, x, cl, normin_y, plans + 0, s))) return rc;
      if ((rc = latrs_dev(true, true, false, n, LU, lda, x, cu, normin_y, plans + 1, s))) return rc;
    } else {                  // inv(U)^T then inv(L)^T
      if ((rc = latrs_dev(true, false, false, n, LU, lda, x, cu, normin_y, plans + 1, s))) return rc;
      if ((rc = latrs_dev(false, false, true, n, LU, lda, x, cl, normin_y, plans + 0, s))) return rc;
    }
    normin_y = true;
    GB_LAUNCH(gecon_rescale_kernel<<<1, 1, 0, s>>>(n, x, plans + 0, plans + 1, stop));
    int hstop = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(&hstop, stop, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hstop) return 0;   // dgecon.f:236: RCOND stays 0
  }
  return 1000 + kStatusCapacity;   // DLACN2 ends within a dozen steps; more means corrupted state
}

int dlatrs_dev(bool upper, bool trans, bool unit, bool normin_y, int n, const double* dA, int lda, double* dX,
               double* scale, double* dCnorm, cudaStream_t s) {
  *scale = 1.0;
  if (n <= 0) return 0;
  DevScratch pb(sizeof(LatrsPlan), s);
  if (!pb.p) return (int)cudaErrorMemoryAllocation;
  LatrsPlan* plan = pb.as<LatrsPlan>();
  int rc = latrs_dev(upper, !trans, unit, n, dA, lda, dX, dCnorm, normin_y, plan, s);
  if (rc) return rc;
  LatrsPlan hp;
  GB_CUDA_TRY(cudaMemcpyAsync(&hp, plan, sizeof(hp), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  *scale = hp.scale;
  return 0;
}

namespace {

// max |A| over the upper triangle (upper) or the whole m x n block, NaN
// propagating, into a host double.
int max_abs_dev(const double* A, int lda, int m, int n, bool upper, double* out, cudaStream_t s) {
  *out = 0.0;
  if (m <= 0 || n <= 0) return 0;
  DevScratch w(16, s);
  if (!w.p) return (int)cudaErrorMemoryAllocation;
  GB_CUDA_TRY(cudaMemsetAsync(w.p, 0, 16, s));
  unsigned long long* bits = w.as<unsigned long long>();
  int* nanflag = reinterpret_cast<int*>(w.as<char>() + 8);
  const size_t tot = (size_t)m * n;
  GB_LAUNCH(max_abs_tri_kernel<<<blocks256(tot), 256, 0, s>>>(A, lda, m, n, upper ? 1 : 0, bits, nanflag));
  unsigned long long hb = 0;
  int hn = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&hb, bits, 8, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(&hn, nanflag, 4, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  double v;
  memcpy(&v, &hb, 8);
  *out = hn ? NAN : v;
  return 0;
}

// RPVGRW of SRC/dgesvx.f:520-545: max|A(:, 1:k)| / max|U(1:k, 1:k)|, 1 when
// the latter is zero.
int rpvgrw_dev(int n, int k, const double* A, int lda, const double* AF, int ldaf, double* out, cudaStream_t s) {
  double u = 0.0, a = 0.0;
  int rc = max_abs_dev(AF, ldaf, k, k, true, &u, s);
  if (rc) return rc;
  if (u == 0.0) {
    *out = 1.0;
    return 0;
  }
  if ((rc = max_abs_dev(A, lda, n, k, false, &a, s))) return rc;
  *out = a / u;
  return 0;
}

}  // namespace

int dgesvx_dev(char fact, char trans, int n, int nrhs, double* A, int lda, double* AF, int ldaf, int* ipiv,
               char* equed, double* R, double* C, double* B, int ldb, double* X, int ldx, double rowcnd,
               double colcnd, double* rcond, double* ferr, double* berr, double* rpvgrw, int* info, cudaStream_t s) {
  // SRC/dgesvx.f:350-597 after the argument checks
  const bool nofact = (fact == 'N' || fact == 'n'), equil = (fact == 'E' || fact == 'e');
  const bool notran = (trans == 'N' || trans == 'n');
  bool rowequ = false, colequ = false;
  if (nofact || equil) {
    *equed = 'N';
  } else {
    rowequ = (*equed == 'R' || *equed == 'r' || *equed == 'B' || *equed == 'b');
    colequ = (*equed == 'C' || *equed == 'c' || *equed == 'B' || *equed == 'b');
  }
  *info = 0;
  *rcond = 0.0;
  *rpvgrw = 1.0;
  int rc;
  if (n == 0) {
    if (nrhs > 0) {
      GB_CUDA_TRY(cudaMemsetAsync(ferr, 0, sizeof(double) * nrhs, s));
      GB_CUDA_TRY(cudaMemsetAsync(berr, 0, sizeof(double) * nrhs, s));
    }
    *rcond = 1.0;   // DGECON's N = 0 answer; RCOND >= eps, so INFO stays 0
    return 0;
  }
  if (equil) {
    // DGEEQU, then DLAQGE's choice (THRESH = 0.1, SMALL = SMLNUM/PREC)
    DevScratch eb(sizeof(EquStat), s);
    if (!eb.p) return (int)cudaErrorMemoryAllocation;
    EquStat* st = eb.as<EquStat>();
    GB_LAUNCH(geequ_rowmax_kernel<<<blocks256(n), 256, 0, s>>>(A, lda, n, n, R));
    GB_LAUNCH(equ_finish_kernel<<<1, 1, 0, s>>>(0, n, n, R, st));
    EquStat hs;
    GB_CUDA_TRY(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hs.info == 0) {
      GB_LAUNCH(geequ_colmax_kernel<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(A, lda, n, n, R, C));
      GB_LAUNCH(equ_finish_kernel<<<1, 1, 0, s>>>(1, n, n, C, st));
      GB_CUDA_TRY(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
      GB_CUDA_TRY(cudaStreamSynchronize(s));
    }
    if (hs.info == 0) {
      rowcnd = hs.rowcnd;
      colcnd = hs.colcnd;
      const double thresh = 0.1, small = kSafeMin / kPrec, large = 1.0 / small;
      const size_t tot = (size_t)n * n;
      if (hs.rowcnd >= thresh && hs.amax >= small && hs.amax <= large) {
        if (hs.colcnd >= thresh) {
          *equed = 'N';
        } else {
          GB_LAUNCH(scale_rows_cols_kernel<<<blocks256(tot), 256, 0, s>>>(A, lda, n, n, nullptr, C));
          *equed = 'C';
        }
      } else if (hs.colcnd >= thresh) {
        GB_LAUNCH(scale_rows_cols_kernel<<<blocks256(tot), 256, 0, s>>>(A, lda, n, n, R, nullptr));
        *equed = 'R';
      } else {
        GB_LAUNCH(scale_rows_cols_kernel<<<blocks256(tot), 256, 0, s>>>(A, lda, n, n, R, C));
        *equed = 'B';
      }
      rowequ = (*equed == 'R' || *equed == 'B');
      colequ = (*equed == 'C' || *equed == 'B');
    }
  }
  const size_t rhs = (size_t)n * nrhs;
  if (nrhs > 0) {
    if (notran && rowequ) GB_LAUNCH(scale_rows_cols_kernel<<<blocks256(rhs), 256, 0, s>>>(B, ldb, n, nrhs, R, nullptr));
    else if (!notran && colequ)
      GB_LAUNCH(scale_rows_cols_kernel<<<blocks256(rhs), 256, 0, s>>>(B, ldb, n, nrhs, C, nullptr));
  }
  if (nofact || equil) {
    GB_CUDA_TRY(cudaMemcpy2DAsync(AF, sizeof(double) * (size_t)ldaf, A, sizeof(double) * (size_t)lda,
                                  sizeof(double) * (size_t)n, n, cudaMemcpyDeviceToDevice, s));
    DevScratch ib(sizeof(int), s);
    if (!ib.p) return (int)cudaErrorMemoryAllocation;
    if ((rc = getrf_dev<double>(n, n, AF, ldaf, ipiv, ib.as<int>(), s, 0, options().nb_f64))) return rc;
    int hinfo = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(&hinfo, ib.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hinfo > 0) {   // dgesvx.f:505-517: singular U, the pivot growth of the leading columns
      *info = hinfo;
      if ((rc = rpvgrw_dev(n, hinfo, A, lda, AF, ldaf, rpvgrw, s))) return rc;
      *rcond = 0.0;
      return 0;
    }
  }
  double anorm = 0.0;
  if ((rc = dlange_dev(notran ? 1 : 2, n, n, A, lda, &anorm, s))) return rc;
  if ((rc = rpvgrw_dev(n, n, A, lda, AF, ldaf, rpvgrw, s))) return rc;
  int cinfo = 0;
  if ((rc = dgecon_dev(notran ? '1' : 'I', n, AF, ldaf, anorm, rcond, &cinfo, s))) return rc;
  if (nrhs > 0) {
    GB_CUDA_TRY(cudaMemcpy2DAsync(X, sizeof(double) * (size_t)ldx, B, sizeof(double) * (size_t)ldb,
                                  sizeof(double) * (size_t)n, nrhs, cudaMemcpyDeviceToDevice, s));
    if ((rc = getrs_dev<double>(notran ? 'N' : 'T', n, nrhs, AF, ldaf, ipiv, nullptr, X, ldx, s))) return rc;
    if ((rc = dgerfs_dev(notran ? 'N' : 'T', n, nrhs, A, lda, AF, ldaf, ipiv, B, ldb, X, ldx, ferr, berr, s)))
      return rc;
    if (notran && colequ) {
      GB_LAUNCH(scale_rows_cols_kernel<<<blocks256(rhs), 256, 0, s>>>(X, ldx, n, nrhs, C, nullptr));
      GB_LAUNCH(div_by_kernel<<<blocks256(nrhs), 256, 0, s>>>(ferr, nrhs, colcnd));
    } else if (!notran && rowequ) {
      GB_LAUNCH(scale_rows_cols_kernel<<<blocks256(rhs), 256, 0, s>>>(X, ldx, n, nrhs, R, nullptr));
      GB_LAUNCH(div_by_kernel<<<blocks256(nrhs), 256, 0, s>>>(ferr, nrhs, rowcnd));
    }
  }
  if (*rcond < 1.1102230246251565e-16) *info = n + 1;   // RCOND < DLAMCH('Epsilon')
  return (int)cudaGetLastError();
}

// FACT = 'F' on device scalings: the MIN <= 0 check and the condition
// number of R (which = 0) or C (which = 1); returns 1 when MIN <= 0.
int scalings_cnd_dev(int n, const double* s_dev, double* cnd, cudaStream_t s, int* err) {
  *err = 0;
  *cnd = 1.0;
  DevScratch b(sizeof(double) + sizeof(int), s);
  if (!b.p) { *err = (int)cudaErrorMemoryAllocation; return 0; }
  double* dc = b.as<double>();
  int* bad = reinterpret_cast<int*>(b.as<char>() + sizeof(double));
  GB_LAUNCH(scalings_cnd_kernel<<<1, 1, 0, s>>>(n, s_dev, dc, bad));
  int hb = 0;
  cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(cnd, dc, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) *err = (int)cudaGetLastError();
  return hb;
}

// DGETRI on device memory (SRC/dgetri.f:169-262): DTRTRI of U by block
// columns of nb_trtri (DTRMM with the inverse so far, DTRSM with the diagonal
// block, DTRTI2 of the diagonal block), then inv(A) from inv(U) and L by block
// columns of nb right to left (DGEMM through the library's update kernel,
// DTRSM with the unit lower block), then the column interchanges.  The two
// block sizes differ as in the reference: DTRTRI always takes its own ILAENV
// value (SRC/dtrtri.f:180, called at SRC/dgetri.f:180), while DGETRI's nb is
// cut to LWORK/N when the workspace is short (SRC/dgetri.f:184-190) and
// nb < 2 selects the unblocked loop.  *info: 0, or the first zero pivot of
// U (A untouched then, as DTRTRI returns before any work).
int dgetri_dev(int n, double* A, int lda, const int* ipiv, int nb_trtri, int nb, int* info, cudaStream_t s) {
  *info = 0;
  if (n <= 0) return 0;
  {
    DevScratch fz(sizeof(int), s);
    if (!fz.p) return (int)cudaErrorMemoryAllocation;
    const int big = 0x7fffffff;
    GB_CUDA_TRY(cudaMemcpyAsync(fz.p, &big, sizeof(int), cudaMemcpyHostToDevice, s));
    GB_LAUNCH(first_zero_diag_kernel<<<blocks256(n), 256, 0, s>>>(A, lda, n, fz.as<int>()));
    int h = big;
    GB_CUDA_TRY(cudaMemcpyAsync(&h, fz.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (h != big) {
      *info = h;
      return 0;
    }
  }
  const int nbt = std::max(1, nb_trtri);
  // ---- DTRTRI('U', 'N')
  if (nbt <= 1 || nbt >= n) {
    GB_LAUNCH(trti2_upper_kernel<<<1, 1, 0, s>>>(n, A, lda));
  } else {
    DevScratch cp(sizeof(double) * (size_t)n * nbt, s);
    if (!cp.p) return (int)cudaErrorMemoryAllocation;
    for (int j = 0; j < n; j += nbt) {
      const int jb = std::min(nbt, n - j);
      double* Bj = A + (size_t)j * lda;   // rows 0..j-1 of block column j
      if (j > 0) {
        GB_CUDA_TRY(cudaMemcpy2DAsync(cp.p, sizeof(double) * (size_t)j, Bj, sizeof(double) * (size_t)lda,
                                      sizeof(double) * (size_t)j, jb, cudaMemcpyDeviceToDevice, s));
        GB_LAUNCH(trmm_lun_kernel<<<blocks256((size_t)j * jb), 256, 0, s>>>(j, jb, A, lda, cp.as<double>(), j, Bj,
                                                                             lda));
        GB_LAUNCH(trsm_rn_kernel<<<blocks256(j), 256, 0, s>>>(j, 1, 1, jb, -1.0, A + j + (size_t)j * lda, lda, Bj,
                                                              lda));
      }
      GB_LAUNCH(trti2_upper_kernel<<<1, 1, 0, s>>>(jb, A + j + (size_t)j * lda, lda));
    }
  }
  // ---- inv(A) * L = inv(U)
  const int nbe = std::max(1, nb);
  const int ldw = n;
  DevScratch wb(sizeof(double) * (size_t)ldw * nbe, s);
  if (!wb.p) return (int)cudaErrorMemoryAllocation;
  double* W = wb.as<double>();
  int rc;
  if (nbe < 2 || nbe >= n) {
    for (int j = n - 1; j >= 0; --j) {
      GB_LAUNCH(getri_take_l_kernel<<<blocks256(n), 256, 0, s>>>(n, j, 1, A, lda, W, ldw));
      if (j < n - 1) GB_LAUNCH(getri_gemv_kernel<<<blocks256(n), 256, 0, s>>>(n, j, A, lda, W));
    }
  } else {
    const int nn = ((n - 1) / nbe) * nbe;
    for (int j = nn; j >= 0; j -= nbe) {
      const int jb = std::min(nbe, n - j);
      GB_LAUNCH(getri_take_l_kernel<<<blocks256((size_t)n * jb), 256, 0, s>>>(n, j, jb, A, lda, W, ldw));
      if (j + jb < n) {
        // A(:, j:j+jb) -= A(:, j+jb:n) * WORK(j+jb:n, 0:jb)   (DGEMM, alpha = -1, beta = 1)
        if ((rc = gemm_update_dev<double>(n, jb, n - j - jb, A + (size_t)(j + jb) * lda, lda, W + j + jb, ldw,
                                          A + (size_t)j * lda, lda, s, 0)))
          return rc;
      }
      GB_LAUNCH(trsm_rn_kernel<<<blocks256(n), 256, 0, s>>>(n, 0, 0, jb, 1.0, W + j, ldw, A + (size_t)j * lda, lda));
    }
  }
  GB_LAUNCH(getri_swap_kernel<<<blocks256(n), 256, 0, s>>>(n, A, lda, ipiv));
  return (int)cudaGetLastError();
}

}  // namespace gb
