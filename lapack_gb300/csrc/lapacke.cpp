// LAPACKE C interface over the Fortran-ABI routines of this library.
// Semantics follow the reference wrappers (LAPACKE/src/lapacke_<name>.c and
// lapacke_<name>_work.c): layout check (-1), optional NaN check of the
// inputs (on by default, LAPACKE_NANCHECK / LAPACKE_set_nancheck), INFO
// shifted by one for the extra layout argument, row-major inputs transposed
// into column-major scratch, IPIV left as the row indices of the transposed
// problem, and the reference's leading-dimension error codes.
#include "../../include/lapack_gb300.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>

namespace {

void* (*g_malloc)(size_t) = malloc;
void (*g_free)(void*) = free;
int g_nancheck = -1;

template <typename T>
bool ge_has_nan(int layout, lapack_int m, lapack_int n, const T* a, lapack_int lda) {
  // LAPACKE/utils/lapacke_dge_nancheck.c: scan min(m, lda) rows of n columns
  // (column major) or min(n, lda) columns of m rows (row major)
  if (!a) return false;
  if (layout == LAPACK_COL_MAJOR) {
    for (lapack_int j = 0; j < n; ++j)
      for (lapack_int i = 0; i < std::min(m, lda); ++i)
        if (a[i + (size_t)j * lda] != a[i + (size_t)j * lda]) return true;
  } else {
    for (lapack_int i = 0; i < m; ++i)
      for (lapack_int j = 0; j < std::min(n, lda); ++j)
        if (a[(size_t)i * lda + j] != a[(size_t)i * lda + j]) return true;
  }
  return false;
}

// Layout change of an m x n matrix given in `layout` (LAPACKE/utils/
// lapacke_dge_trans.c): out(j, i) = in(i, j), clipped by the leading
// dimensions exactly as the reference does.
template <typename T>
void ge_trans(int layout, lapack_int m, lapack_int n, const T* in, lapack_int ldin, T* out, lapack_int ldout) {
  if (!in || !out) return;
  lapack_int x, y;
  if (layout == LAPACK_COL_MAJOR) { x = n; y = m; }
  else if (layout == LAPACK_ROW_MAJOR) { x = m; y = n; }
  else return;
  for (lapack_int i = 0; i < std::min(y, ldin); ++i)
    for (lapack_int j = 0; j < std::min(x, ldout); ++j) out[(size_t)i * ldout + j] = in[(size_t)j * ldin + i];
}

template <typename T>
T* alloc(size_t count) { return static_cast<T*>(LAPACKE_malloc_proxy(sizeof(T) * std::max<size_t>(1, count))); }

bool nancheck() { return LAPACKE_get_nancheck() != 0; }

// ---- GESV
template <typename T, typename F>
lapack_int gesv_work(const char* nm, F fort, int layout, lapack_int n, lapack_int nrhs, T* a, lapack_int lda,
                     lapack_int* ipiv, T* b, lapack_int ldb) {
  lapack_int info = 0;
  if (layout == LAPACK_COL_MAJOR) {
    fort(&n, &nrhs, a, &lda, ipiv, b, &ldb, &info);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n), ldb_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -5); return -5; }
  if (ldb < nrhs) { LAPACKE_xerbla(nm, -8); return -8; }
  T* a_t = alloc<T>((size_t)lda_t * std::max(1, n));
  if (!a_t) { LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR); return LAPACK_TRANSPOSE_MEMORY_ERROR; }
  T* b_t = alloc<T>((size_t)ldb_t * std::max(1, nrhs));
  if (!b_t) { LAPACKE_free_proxy(a_t); LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR); return LAPACK_TRANSPOSE_MEMORY_ERROR; }
  ge_trans(layout, n, n, a, lda, a_t, lda_t);
  ge_trans(layout, n, nrhs, b, ldb, b_t, ldb_t);
  fort(&n, &nrhs, a_t, &lda_t, ipiv, b_t, &ldb_t, &info);
  if (info < 0) info -= 1;
  ge_trans(LAPACK_COL_MAJOR, n, n, a_t, lda_t, a, lda);
  ge_trans(LAPACK_COL_MAJOR, n, nrhs, b_t, ldb_t, b, ldb);
  LAPACKE_free_proxy(b_t);
  LAPACKE_free_proxy(a_t);
  return info;
}

// ---- GETRF / GETRF2
template <typename T, typename F>
lapack_int getrf_work(const char* nm, F fort, int layout, lapack_int m, lapack_int n, T* a, lapack_int lda,
                      lapack_int* ipiv) {
  lapack_int info = 0;
  if (layout == LAPACK_COL_MAJOR) {
    fort(&m, &n, a, &lda, ipiv, &info);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, m);
  if (lda < n) { LAPACKE_xerbla(nm, -5); return -5; }
  T* a_t = alloc<T>((size_t)lda_t * std::max(1, n));
  if (!a_t) { LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR); return LAPACK_TRANSPOSE_MEMORY_ERROR; }
  ge_trans(layout, m, n, a, lda, a_t, lda_t);
  fort(&m, &n, a_t, &lda_t, ipiv, &info);
  if (info < 0) info -= 1;
  ge_trans(LAPACK_COL_MAJOR, m, n, a_t, lda_t, a, lda);
  LAPACKE_free_proxy(a_t);
  return info;
}

// ---- GETRS
template <typename T, typename F>
lapack_int getrs_work(const char* nm, F fort, int layout, char trans, lapack_int n, lapack_int nrhs, const T* a,
                      lapack_int lda, const lapack_int* ipiv, T* b, lapack_int ldb) {
  lapack_int info = 0;
  if (layout == LAPACK_COL_MAJOR) {
    fort(&trans, &n, &nrhs, a, &lda, ipiv, b, &ldb, &info, 1);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n), ldb_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -6); return -6; }
  if (ldb < nrhs) { LAPACKE_xerbla(nm, -9); return -9; }
  T* a_t = alloc<T>((size_t)lda_t * std::max(1, n));
  if (!a_t) { LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR); return LAPACK_TRANSPOSE_MEMORY_ERROR; }
  T* b_t = alloc<T>((size_t)ldb_t * std::max(1, nrhs));
  if (!b_t) { LAPACKE_free_proxy(a_t); LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR); return LAPACK_TRANSPOSE_MEMORY_ERROR; }
  ge_trans(layout, n, n, a, lda, a_t, lda_t);
  ge_trans(layout, n, nrhs, b, ldb, b_t, ldb_t);
  fort(&trans, &n, &nrhs, a_t, &lda_t, ipiv, b_t, &ldb_t, &info, 1);
  if (info < 0) info -= 1;
  ge_trans(LAPACK_COL_MAJOR, n, nrhs, b_t, ldb_t, b, ldb);
  LAPACKE_free_proxy(b_t);
  LAPACKE_free_proxy(a_t);
  return info;
}

// ---- LASWP
template <typename T, typename F>
lapack_int laswp_work(const char* nm, F fort, int layout, lapack_int n, T* a, lapack_int lda, lapack_int k1,
                      lapack_int k2, const lapack_int* ipiv, lapack_int incx) {
  if (layout == LAPACK_COL_MAJOR) {
    fort(&n, a, &lda, &k1, &k2, ipiv, &incx);
    return 0;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  // rows referenced: up to K2 and every IPIV target (LAPACKE/src/lapacke_dlaswp_work.c)
  lapack_int lda_t = std::max(1, k2);
  for (lapack_int i = k1; i <= k2; ++i) lda_t = std::max(lda_t, ipiv[k1 + (i - k1) * std::abs(incx) - 1]);
  if (lda < n) { LAPACKE_xerbla(nm, -4); return -4; }
  T* a_t = alloc<T>((size_t)lda_t * std::max(1, n));
  if (!a_t) { LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR); return LAPACK_TRANSPOSE_MEMORY_ERROR; }
  ge_trans(layout, lda_t, n, a, lda, a_t, lda_t);
  fort(&n, a_t, &lda_t, &k1, &k2, ipiv, &incx);
  ge_trans(LAPACK_COL_MAJOR, lda_t, n, a_t, lda_t, a, lda);
  LAPACKE_free_proxy(a_t);
  return 0;
}


// NaN check of the UPLO triangle (LAPACKE/utils/lapacke_dtr_nancheck.c with
// DIAG = 'N', as LAPACKE_dpo_nancheck calls it): the triangle of the stored
// matrix in the given layout, clipped by LDA.
template <typename T>
bool tr_has_nan(int layout, char uplo, lapack_int n, const T* a, lapack_int lda) {
  if (!a) return false;
  const bool colmaj = layout == LAPACK_COL_MAJOR, lower = (uplo | 0x20) == 'l';
  if ((!colmaj && layout != LAPACK_ROW_MAJOR) || (!lower && (uplo | 0x20) != 'u')) return false;
  if (colmaj != lower) {   // column-major upper or row-major lower
    for (lapack_int j = 0; j < n; ++j)
      for (lapack_int i = 0; i < std::min(j + 1, lda); ++i)
        if (a[i + (size_t)j * lda] != a[i + (size_t)j * lda]) return true;
  } else {
    for (lapack_int j = 0; j < n; ++j)
      for (lapack_int i = j; i < std::min(n, lda); ++i)
        if (a[i + (size_t)j * lda] != a[i + (size_t)j * lda]) return true;
  }
  return false;
}

// Layout change of the UPLO triangle (LAPACKE/utils/lapacke_dtr_trans.c with
// DIAG = 'N'): out(j, i) = in(i, j) over the triangle, clipped by both
// leading dimensions; the other triangle of `out` is not written.
template <typename T>
void tr_trans(int layout, char uplo, lapack_int n, const T* in, lapack_int ldin, T* out, lapack_int ldout) {
  if (!in || !out) return;
  const bool colmaj = layout == LAPACK_COL_MAJOR, lower = (uplo | 0x20) == 'l';
  if ((!colmaj && layout != LAPACK_ROW_MAJOR) || (!lower && (uplo | 0x20) != 'u')) return;
  if (colmaj != lower) {
    for (lapack_int j = 0; j < std::min(n, ldout); ++j)
      for (lapack_int i = 0; i < std::min(j + 1, ldin); ++i) out[j + (size_t)i * ldout] = in[i + (size_t)j * ldin];
  } else {
    for (lapack_int j = 0; j < std::min(n, ldout); ++j)
      for (lapack_int i = j; i < std::min(n, ldin); ++i) out[j + (size_t)i * ldout] = in[i + (size_t)j * ldin];
  }
}

// ---- POTRF / POTRS / POSV (LAPACKE/src/lapacke_dpotrf*.c, dpotrs*.c, dposv*.c)
template <typename T, typename F>
lapack_int potrf_work(const char* nm, F fort, int layout, char uplo, lapack_int n, T* a, lapack_int lda) {
  lapack_int info = 0;
  if (layout == LAPACK_COL_MAJOR) {
    fort(&uplo, &n, a, &lda, &info, 1);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -5); return -5; }
  T* a_t = alloc<T>((size_t)lda_t * std::max(1, n));
  if (!a_t) { LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR); return LAPACK_TRANSPOSE_MEMORY_ERROR; }
  tr_trans(layout, uplo, n, a, lda, a_t, lda_t);
  fort(&uplo, &n, a_t, &lda_t, &info, 1);
  if (info < 0) info -= 1;
  tr_trans(LAPACK_COL_MAJOR, uplo, n, a_t, lda_t, a, lda);
  LAPACKE_free_proxy(a_t);
  return info;
}
// potrs (solve only, A not written back) and posv (factor written back)
template <typename T, typename F>
lapack_int potrs_posv_work(const char* nm, F fort, bool write_a, int layout, char uplo, lapack_int n, lapack_int nrhs,
                           T* a, lapack_int lda, T* b, lapack_int ldb) {
  lapack_int info = 0;
  if (layout == LAPACK_COL_MAJOR) {
    fort(&uplo, &n, &nrhs, a, &lda, b, &ldb, &info, 1);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n), ldb_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -6); return -6; }
  if (ldb < nrhs) { LAPACKE_xerbla(nm, -8); return -8; }
  T* a_t = alloc<T>((size_t)lda_t * std::max(1, n));
  T* b_t = a_t ? alloc<T>((size_t)ldb_t * std::max(1, nrhs)) : nullptr;
  if (!b_t) {
    if (a_t) LAPACKE_free_proxy(a_t);
    LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR);
    return LAPACK_TRANSPOSE_MEMORY_ERROR;
  }
  tr_trans(layout, uplo, n, a, lda, a_t, lda_t);
  ge_trans(layout, n, nrhs, b, ldb, b_t, ldb_t);
  fort(&uplo, &n, &nrhs, a_t, &lda_t, b_t, &ldb_t, &info, 1);
  if (info < 0) info -= 1;
  if (write_a) tr_trans(LAPACK_COL_MAJOR, uplo, n, a_t, lda_t, a, lda);
  ge_trans(LAPACK_COL_MAJOR, n, nrhs, b_t, ldb_t, b, ldb);
  LAPACKE_free_proxy(b_t);
  LAPACKE_free_proxy(a_t);
  return info;
}

// COMPLEX*16 / COMPLEX elements for the generic wrappers above: x != x
// holds when either part is a NaN (LAPACKE/utils/lapacke_zge_nancheck.c
// through LAPACKE_zisnan).
struct zc_t {
  double re, im;
  bool operator!=(const zc_t& o) const { return re != o.re || im != o.im; }
};
struct cc_t {
  float re, im;
  bool operator!=(const cc_t& o) const { return re != o.re || im != o.im; }
};

}  // namespace

extern "C" {

void* LAPACKE_malloc_proxy(size_t size) { return g_malloc(size); }
void LAPACKE_free_proxy(void* ptr) { g_free(ptr); }
void LAPACKE_set_alloc(void* (*malloc_fn)(size_t), void (*free_fn)(void*)) {
  g_malloc = malloc_fn ? malloc_fn : malloc;
  g_free = free_fn ? free_fn : free;
}

void LAPACKE_set_nancheck(int flag) { g_nancheck = flag ? 1 : 0; }
int LAPACKE_get_nancheck(void) {
  if (g_nancheck != -1) return g_nancheck;
  const char* env = getenv("LAPACKE_NANCHECK");   // read once; enabled unless set to 0
  g_nancheck = env ? (atoi(env) ? 1 : 0) : 1;
  return g_nancheck;
}

void LAPACKE_xerbla(const char* name, lapack_int info) {
  // LAPACKE/utils/lapacke_xerbla.c messages
  if (info == LAPACK_WORK_MEMORY_ERROR) printf("Not enough memory to allocate work array in %s\n", name);
  else if (info == LAPACK_TRANSPOSE_MEMORY_ERROR) printf("Not enough memory to transpose matrix in %s\n", name);
  else if (info < 0) printf("Wrong parameter %d in %s\n", -(int)info, name);
}

// ---------------------------------------------------------------- GESV
lapack_int LAPACKE_dgesv_work(int layout, lapack_int n, lapack_int nrhs, double* a, lapack_int lda, lapack_int* ipiv,
                              double* b, lapack_int ldb) {
  return gesv_work<double>("LAPACKE_dgesv_work", dgesv_, layout, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_sgesv_work(int layout, lapack_int n, lapack_int nrhs, float* a, lapack_int lda, lapack_int* ipiv,
                              float* b, lapack_int ldb) {
  return gesv_work<float>("LAPACKE_sgesv_work", sgesv_, layout, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_dgesv(int layout, lapack_int n, lapack_int nrhs, double* a, lapack_int lda, lapack_int* ipiv,
                         double* b, lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dgesv", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, a, lda)) return -4;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -7;
  }
  return LAPACKE_dgesv_work(layout, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_sgesv(int layout, lapack_int n, lapack_int nrhs, float* a, lapack_int lda, lapack_int* ipiv,
                         float* b, lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_sgesv", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, a, lda)) return -4;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -7;
  }
  return LAPACKE_sgesv_work(layout, n, nrhs, a, lda, ipiv, b, ldb);
}

// ---------------------------------------------------------------- GETRF
lapack_int LAPACKE_dgetrf_work(int layout, lapack_int m, lapack_int n, double* a, lapack_int lda, lapack_int* ipiv) {
  return getrf_work<double>("LAPACKE_dgetrf_work", dgetrf_, layout, m, n, a, lda, ipiv);
}
lapack_int LAPACKE_dgetrf2_work(int layout, lapack_int m, lapack_int n, double* a, lapack_int lda, lapack_int* ipiv) {
  return getrf_work<double>("LAPACKE_dgetrf2_work", dgetrf2_, layout, m, n, a, lda, ipiv);
}
lapack_int LAPACKE_sgetrf_work(int layout, lapack_int m, lapack_int n, float* a, lapack_int lda, lapack_int* ipiv) {
  return getrf_work<float>("LAPACKE_sgetrf_work", sgetrf_, layout, m, n, a, lda, ipiv);
}
lapack_int LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double* a, lapack_int lda, lapack_int* ipiv) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dgetrf", -1); return -1; }
  if (nancheck() && ge_has_nan(layout, m, n, a, lda)) return -4;
  return LAPACKE_dgetrf_work(layout, m, n, a, lda, ipiv);
}
lapack_int LAPACKE_dgetrf2(int layout, lapack_int m, lapack_int n, double* a, lapack_int lda, lapack_int* ipiv) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dgetrf2", -1); return -1; }
  if (nancheck() && ge_has_nan(layout, m, n, a, lda)) return -4;
  return LAPACKE_dgetrf2_work(layout, m, n, a, lda, ipiv);
}
lapack_int LAPACKE_sgetrf(int layout, lapack_int m, lapack_int n, float* a, lapack_int lda, lapack_int* ipiv) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_sgetrf", -1); return -1; }
  if (nancheck() && ge_has_nan(layout, m, n, a, lda)) return -4;
  return LAPACKE_sgetrf_work(layout, m, n, a, lda, ipiv);
}

// ---------------------------------------------------------------- GETRS
lapack_int LAPACKE_dgetrs_work(int layout, char trans, lapack_int n, lapack_int nrhs, const double* a, lapack_int lda,
                               const lapack_int* ipiv, double* b, lapack_int ldb) {
  return getrs_work<double>("LAPACKE_dgetrs_work", dgetrs_, layout, trans, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_sgetrs_work(int layout, char trans, lapack_int n, lapack_int nrhs, const float* a, lapack_int lda,
                               const lapack_int* ipiv, float* b, lapack_int ldb) {
  return getrs_work<float>("LAPACKE_sgetrs_work", sgetrs_, layout, trans, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_dgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const double* a, lapack_int lda,
                          const lapack_int* ipiv, double* b, lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dgetrs", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, a, lda)) return -5;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -8;
  }
  return LAPACKE_dgetrs_work(layout, trans, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_sgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const float* a, lapack_int lda,
                          const lapack_int* ipiv, float* b, lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_sgetrs", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, a, lda)) return -5;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -8;
  }
  return LAPACKE_sgetrs_work(layout, trans, n, nrhs, a, lda, ipiv, b, ldb);
}

// ---------------------------------------------------------------- DSGESV
lapack_int LAPACKE_dsgesv_work(int layout, lapack_int n, lapack_int nrhs, double* a, lapack_int lda, lapack_int* ipiv,
                               const double* b, lapack_int ldb, double* x, lapack_int ldx, double* work, float* swork,
                               lapack_int* iter) {
  lapack_int info = 0;
  const char* nm = "LAPACKE_dsgesv_work";
  if (layout == LAPACK_COL_MAJOR) {
    dsgesv_(&n, &nrhs, a, &lda, ipiv, b, &ldb, x, &ldx, work, swork, iter, &info);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n), ldb_t = std::max(1, n), ldx_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -5); return -5; }
  if (ldb < nrhs) { LAPACKE_xerbla(nm, -8); return -8; }
  if (ldx < nrhs) { LAPACKE_xerbla(nm, -10); return -10; }
  double* a_t = alloc<double>((size_t)lda_t * std::max(1, n));
  double* b_t = a_t ? alloc<double>((size_t)ldb_t * std::max(1, nrhs)) : nullptr;
  double* x_t = b_t ? alloc<double>((size_t)ldx_t * std::max(1, nrhs)) : nullptr;
  if (!x_t) {
    if (b_t) LAPACKE_free_proxy(b_t);
    if (a_t) LAPACKE_free_proxy(a_t);
    LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR);
    return LAPACK_TRANSPOSE_MEMORY_ERROR;
  }
  ge_trans(layout, n, n, a, lda, a_t, lda_t);
  ge_trans(layout, n, nrhs, b, ldb, b_t, ldb_t);
  dsgesv_(&n, &nrhs, a_t, &lda_t, ipiv, b_t, &ldb_t, x_t, &ldx_t, work, swork, iter, &info);
  if (info < 0) info -= 1;
  ge_trans(LAPACK_COL_MAJOR, n, n, a_t, lda_t, a, lda);
  ge_trans(LAPACK_COL_MAJOR, n, nrhs, x_t, ldx_t, x, ldx);
  LAPACKE_free_proxy(x_t);
  LAPACKE_free_proxy(b_t);
  LAPACKE_free_proxy(a_t);
  return info;
}
lapack_int LAPACKE_dsgesv(int layout, lapack_int n, lapack_int nrhs, double* a, lapack_int lda, lapack_int* ipiv,
                          const double* b, lapack_int ldb, double* x, lapack_int ldx, lapack_int* iter) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dsgesv", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, a, lda)) return -4;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -7;
  }
  // WORK / SWORK as LAPACKE_dsgesv sizes them (LAPACKE/src/lapacke_dsgesv.c:59-68)
  float* swork = alloc<float>((size_t)std::max(1, n) * std::max(1, n + nrhs));
  double* work = swork ? alloc<double>((size_t)std::max(1, n) * std::max(1, nrhs)) : nullptr;
  if (!work) {
    if (swork) LAPACKE_free_proxy(swork);
    LAPACKE_xerbla("LAPACKE_dsgesv", LAPACK_WORK_MEMORY_ERROR);
    return LAPACK_WORK_MEMORY_ERROR;
  }
  lapack_int info = LAPACKE_dsgesv_work(layout, n, nrhs, a, lda, ipiv, b, ldb, x, ldx, work, swork, iter);
  LAPACKE_free_proxy(work);
  LAPACKE_free_proxy(swork);
  return info;
}

// ---------------------------------------------------------------- LASWP
lapack_int LAPACKE_dlaswp_work(int layout, lapack_int n, double* a, lapack_int lda, lapack_int k1, lapack_int k2,
                               const lapack_int* ipiv, lapack_int incx) {
  return laswp_work<double>("LAPACKE_dlaswp_work", dlaswp_, layout, n, a, lda, k1, k2, ipiv, incx);
}
lapack_int LAPACKE_slaswp_work(int layout, lapack_int n, float* a, lapack_int lda, lapack_int k1, lapack_int k2,
                               const lapack_int* ipiv, lapack_int incx) {
  return laswp_work<float>("LAPACKE_slaswp_work", slaswp_, layout, n, a, lda, k1, k2, ipiv, incx);
}
lapack_int LAPACKE_dlaswp(int layout, lapack_int n, double* a, lapack_int lda, lapack_int k1, lapack_int k2,
                          const lapack_int* ipiv, lapack_int incx) {
  // the reference disables the NaN check of DLASWP (LAPACKE/src/lapacke_dlaswp.c:44-58)
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dlaswp", -1); return -1; }
  return LAPACKE_dlaswp_work(layout, n, a, lda, k1, k2, ipiv, incx);
}
lapack_int LAPACKE_slaswp(int layout, lapack_int n, float* a, lapack_int lda, lapack_int k1, lapack_int k2,
                          const lapack_int* ipiv, lapack_int incx) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_slaswp", -1); return -1; }
  return LAPACKE_slaswp_work(layout, n, a, lda, k1, k2, ipiv, incx);
}

// ---------------------------------------------------------------- LAG2S / LAG2D
lapack_int LAPACKE_dlag2s_work(int layout, lapack_int m, lapack_int n, const double* a, lapack_int lda, float* sa,
                               lapack_int ldsa) {
  lapack_int info = 0;
  const char* nm = "LAPACKE_dlag2s_work";
  if (layout == LAPACK_COL_MAJOR) {
    dlag2s_(&m, &n, a, &lda, sa, &ldsa, &info);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, m), ldsa_t = std::max(1, m);
  if (lda < n) { LAPACKE_xerbla(nm, -5); return -5; }
  if (ldsa < n) { LAPACKE_xerbla(nm, -7); return -7; }
  double* a_t = alloc<double>((size_t)lda_t * std::max(1, n));
  float* sa_t = a_t ? alloc<float>((size_t)ldsa_t * std::max(1, n)) : nullptr;
  if (!sa_t) {
    if (a_t) LAPACKE_free_proxy(a_t);
    LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR);
    return LAPACK_TRANSPOSE_MEMORY_ERROR;
  }
  ge_trans(layout, m, n, a, lda, a_t, lda_t);
  dlag2s_(&m, &n, a_t, &lda_t, sa_t, &ldsa_t, &info);
  if (info < 0) info -= 1;
  ge_trans(LAPACK_COL_MAJOR, m, n, sa_t, ldsa_t, sa, ldsa);
  LAPACKE_free_proxy(sa_t);
  LAPACKE_free_proxy(a_t);
  return info;
}
lapack_int LAPACKE_dlag2s(int layout, lapack_int m, lapack_int n, const double* a, lapack_int lda, float* sa,
                          lapack_int ldsa) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dlag2s", -1); return -1; }
  if (nancheck() && ge_has_nan(layout, m, n, a, lda)) return -4;
  return LAPACKE_dlag2s_work(layout, m, n, a, lda, sa, ldsa);
}
lapack_int LAPACKE_slag2d_work(int layout, lapack_int m, lapack_int n, const float* sa, lapack_int ldsa, double* a,
                               lapack_int lda) {
  lapack_int info = 0;
  const char* nm = "LAPACKE_slag2d_work";
  if (layout == LAPACK_COL_MAJOR) {
    slag2d_(&m, &n, sa, &ldsa, a, &lda, &info);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int ldsa_t = std::max(1, m), lda_t = std::max(1, m);
  if (lda < n) { LAPACKE_xerbla(nm, -7); return -7; }
  if (ldsa < n) { LAPACKE_xerbla(nm, -5); return -5; }
  float* sa_t = alloc<float>((size_t)ldsa_t * std::max(1, n));
  double* a_t = sa_t ? alloc<double>((size_t)lda_t * std::max(1, n)) : nullptr;
  if (!a_t) {
    if (sa_t) LAPACKE_free_proxy(sa_t);
    LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR);
    return LAPACK_TRANSPOSE_MEMORY_ERROR;
  }
  ge_trans(layout, m, n, sa, ldsa, sa_t, ldsa_t);
  slag2d_(&m, &n, sa_t, &ldsa_t, a_t, &lda_t, &info);
  if (info < 0) info -= 1;
  ge_trans(LAPACK_COL_MAJOR, m, n, a_t, lda_t, a, lda);
  LAPACKE_free_proxy(a_t);
  LAPACKE_free_proxy(sa_t);
  return info;
}
lapack_int LAPACKE_slag2d(int layout, lapack_int m, lapack_int n, const float* sa, lapack_int ldsa, double* a,
                          lapack_int lda) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_slag2d", -1); return -1; }
  if (nancheck() && ge_has_nan(layout, m, n, sa, ldsa)) return -4;
  return LAPACKE_slag2d_work(layout, m, n, sa, ldsa, a, lda);
}

// ---------------------------------------------------------------- GECON
// LAPACKE/src/lapacke_dgecon.c, lapacke_dgecon_work.c: NaN checks of A (-4)
// and ANORM (-6); row-major A transposed into scratch (LDA < N: -5).
lapack_int LAPACKE_dgecon_work(int layout, char norm, lapack_int n, const double* a, lapack_int lda, double anorm,
                               double* rcond, double* work, lapack_int* iwork) {
  lapack_int info = 0;
  const char* nm = "LAPACKE_dgecon_work";
  if (layout == LAPACK_COL_MAJOR) {
    dgecon_(&norm, &n, a, &lda, &anorm, rcond, work, iwork, &info, 1);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -5); return -5; }
  double* a_t = alloc<double>((size_t)lda_t * std::max(1, n));
  if (!a_t) { LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR); return LAPACK_TRANSPOSE_MEMORY_ERROR; }
  ge_trans(layout, n, n, a, lda, a_t, lda_t);
  dgecon_(&norm, &n, a_t, &lda_t, &anorm, rcond, work, iwork, &info, 1);
  if (info < 0) info -= 1;
  LAPACKE_free_proxy(a_t);
  return info;
}
lapack_int LAPACKE_dgecon(int layout, char norm, lapack_int n, const double* a, lapack_int lda, double anorm,
                          double* rcond) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dgecon", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, a, lda)) return -4;
    if (anorm != anorm) return -6;
  }
  lapack_int* iwork = alloc<lapack_int>((size_t)std::max(1, n));
  double* work = iwork ? alloc<double>((size_t)std::max(1, 4 * n)) : nullptr;
  if (!work) {
    if (iwork) LAPACKE_free_proxy(iwork);
    LAPACKE_xerbla("LAPACKE_dgecon", LAPACK_WORK_MEMORY_ERROR);
    return LAPACK_WORK_MEMORY_ERROR;
  }
  lapack_int info = LAPACKE_dgecon_work(layout, norm, n, a, lda, anorm, rcond, work, iwork);
  LAPACKE_free_proxy(work);
  LAPACKE_free_proxy(iwork);
  return info;
}

// ---------------------------------------------------------------- GERFS
// LAPACKE/src/lapacke_dgerfs.c, lapacke_dgerfs_work.c: NaN checks of A (-5),
// AF (-7), B (-10), X (-12); row-major: LDA, LDAF < N give -6, -8, LDB,
// LDX < NRHS give -11, -13; only X is transposed back.
lapack_int LAPACKE_dgerfs_work(int layout, char trans, lapack_int n, lapack_int nrhs, const double* a,
                               lapack_int lda, const double* af, lapack_int ldaf, const lapack_int* ipiv,
                               const double* b, lapack_int ldb, double* x, lapack_int ldx, double* ferr,
                               double* berr, double* work, lapack_int* iwork) {
  lapack_int info = 0;
  const char* nm = "LAPACKE_dgerfs_work";
  if (layout == LAPACK_COL_MAJOR) {
    dgerfs_(&trans, &n, &nrhs, a, &lda, af, &ldaf, ipiv, b, &ldb, x, &ldx, ferr, berr, work, iwork, &info, 1);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n), ldaf_t = std::max(1, n), ldb_t = std::max(1, n), ldx_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -6); return -6; }
  if (ldaf < n) { LAPACKE_xerbla(nm, -8); return -8; }
  if (ldb < nrhs) { LAPACKE_xerbla(nm, -11); return -11; }
  if (ldx < nrhs) { LAPACKE_xerbla(nm, -13); return -13; }
  double* a_t = alloc<double>((size_t)lda_t * std::max(1, n));
  double* af_t = a_t ? alloc<double>((size_t)ldaf_t * std::max(1, n)) : nullptr;
  double* b_t = af_t ? alloc<double>((size_t)ldb_t * std::max(1, nrhs)) : nullptr;
  double* x_t = b_t ? alloc<double>((size_t)ldx_t * std::max(1, nrhs)) : nullptr;
  if (!x_t) {
    if (b_t) LAPACKE_free_proxy(b_t);
    if (af_t) LAPACKE_free_proxy(af_t);
    if (a_t) LAPACKE_free_proxy(a_t);
    LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR);
    return LAPACK_TRANSPOSE_MEMORY_ERROR;
  }
  ge_trans(layout, n, n, a, lda, a_t, lda_t);
  ge_trans(layout, n, n, af, ldaf, af_t, ldaf_t);
  ge_trans(layout, n, nrhs, b, ldb, b_t, ldb_t);
  ge_trans(layout, n, nrhs, x, ldx, x_t, ldx_t);
  dgerfs_(&trans, &n, &nrhs, a_t, &lda_t, af_t, &ldaf_t, ipiv, b_t, &ldb_t, x_t, &ldx_t, ferr, berr, work, iwork,
          &info, 1);
  if (info < 0) info -= 1;
  ge_trans(LAPACK_COL_MAJOR, n, nrhs, x_t, ldx_t, x, ldx);
  LAPACKE_free_proxy(x_t);
  LAPACKE_free_proxy(b_t);
  LAPACKE_free_proxy(af_t);
  LAPACKE_free_proxy(a_t);
  return info;
}
lapack_int LAPACKE_dgerfs(int layout, char trans, lapack_int n, lapack_int nrhs, const double* a, lapack_int lda,
                          const double* af, lapack_int ldaf, const lapack_int* ipiv, const double* b, lapack_int ldb,
                          double* x, lapack_int ldx, double* ferr, double* berr) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dgerfs", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, a, lda)) return -5;
    if (ge_has_nan(layout, n, n, af, ldaf)) return -7;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -10;
    if (ge_has_nan(layout, n, nrhs, x, ldx)) return -12;
  }
  lapack_int* iwork = alloc<lapack_int>((size_t)std::max(1, n));
  double* work = iwork ? alloc<double>((size_t)std::max(1, 3 * n)) : nullptr;
  if (!work) {
    if (iwork) LAPACKE_free_proxy(iwork);
    LAPACKE_xerbla("LAPACKE_dgerfs", LAPACK_WORK_MEMORY_ERROR);
    return LAPACK_WORK_MEMORY_ERROR;
  }
  lapack_int info = LAPACKE_dgerfs_work(layout, trans, n, nrhs, a, lda, af, ldaf, ipiv, b, ldb, x, ldx, ferr, berr,
                                        work, iwork);
  LAPACKE_free_proxy(work);
  LAPACKE_free_proxy(iwork);
  return info;
}

// ---------------------------------------------------------------- GESVX
// LAPACKE/src/lapacke_dgesvx.c, lapacke_dgesvx_work.c.  NaN checks: A (-6),
// AF when FACT = 'F' (-8), B (-14), C (-13) when FACT = 'F' and EQUED is
// 'B' or 'C', R (-12) when FACT = 'F' and EQUED is 'B' or 'R'.  Row major:
// LDA, LDAF < N give -7, -9, LDB, LDX < NRHS give -15, -17; AF is
// transposed in only for FACT = 'F'; written back are A when FACT = 'E'
// and EQUED != 'N', AF when FACT is 'E' or 'N', B when FACT = 'F' and
// EQUED != 'N', and X.  WORK(1) (the reciprocal pivot growth) is returned
// in *rpivot.
namespace {
bool lsame_c(char a, char b) { return (a | 0x20) == (b | 0x20); }
bool vec_has_nan(lapack_int n, const double* x) {
  for (lapack_int i = 0; i < n; ++i)
    if (x[i] != x[i]) return true;
  return false;
}
}  // namespace

lapack_int LAPACKE_dgesvx_work(int layout, char fact, char trans, lapack_int n, lapack_int nrhs, double* a,
                               lapack_int lda, double* af, lapack_int ldaf, lapack_int* ipiv, char* equed, double* r,
                               double* c, double* b, lapack_int ldb, double* x, lapack_int ldx, double* rcond,
                               double* ferr, double* berr, double* work, lapack_int* iwork) {
  lapack_int info = 0;
  const char* nm = "LAPACKE_dgesvx_work";
  if (layout == LAPACK_COL_MAJOR) {
    dgesvx_(&fact, &trans, &n, &nrhs, a, &lda, af, &ldaf, ipiv, equed, r, c, b, &ldb, x, &ldx, rcond, ferr, berr,
            work, iwork, &info, 1, 1, 1);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n), ldaf_t = std::max(1, n), ldb_t = std::max(1, n), ldx_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -7); return -7; }
  if (ldaf < n) { LAPACKE_xerbla(nm, -9); return -9; }
  if (ldb < nrhs) { LAPACKE_xerbla(nm, -15); return -15; }
  if (ldx < nrhs) { LAPACKE_xerbla(nm, -17); return -17; }
  double* a_t = alloc<double>((size_t)lda_t * std::max(1, n));
  double* af_t = a_t ? alloc<double>((size_t)ldaf_t * std::max(1, n)) : nullptr;
  double* b_t = af_t ? alloc<double>((size_t)ldb_t * std::max(1, nrhs)) : nullptr;
  double* x_t = b_t ? alloc<double>((size_t)ldx_t * std::max(1, nrhs)) : nullptr;
  if (!x_t) {
    if (b_t) LAPACKE_free_proxy(b_t);
    if (af_t) LAPACKE_free_proxy(af_t);
    if (a_t) LAPACKE_free_proxy(a_t);
    LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR);
    return LAPACK_TRANSPOSE_MEMORY_ERROR;
  }
  ge_trans(layout, n, n, a, lda, a_t, lda_t);
  if (lsame_c(fact, 'f')) ge_trans(layout, n, n, af, ldaf, af_t, ldaf_t);
  ge_trans(layout, n, nrhs, b, ldb, b_t, ldb_t);
  dgesvx_(&fact, &trans, &n, &nrhs, a_t, &lda_t, af_t, &ldaf_t, ipiv, equed, r, c, b_t, &ldb_t, x_t, &ldx_t, rcond,
          ferr, berr, work, iwork, &info, 1, 1, 1);
  if (info < 0) info -= 1;
  const bool scaled = lsame_c(*equed, 'b') || lsame_c(*equed, 'c') || lsame_c(*equed, 'r');
  if (lsame_c(fact, 'e') && scaled) ge_trans(LAPACK_COL_MAJOR, n, n, a_t, lda_t, a, lda);
  if (lsame_c(fact, 'e') || lsame_c(fact, 'n')) ge_trans(LAPACK_COL_MAJOR, n, n, af_t, ldaf_t, af, ldaf);
  if (lsame_c(fact, 'f') && scaled) ge_trans(LAPACK_COL_MAJOR, n, nrhs, b_t, ldb_t, b, ldb);
  ge_trans(LAPACK_COL_MAJOR, n, nrhs, x_t, ldx_t, x, ldx);
  LAPACKE_free_proxy(x_t);
  LAPACKE_free_proxy(b_t);
  LAPACKE_free_proxy(af_t);
  LAPACKE_free_proxy(a_t);
  return info;
}
lapack_int LAPACKE_dgesvx(int layout, char fact, char trans, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                          double* af, lapack_int ldaf, lapack_int* ipiv, char* equed, double* r, double* c, double* b,
                          lapack_int ldb, double* x, lapack_int ldx, double* rcond, double* ferr, double* berr,
                          double* rpivot) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dgesvx", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, a, lda)) return -6;
    if (lsame_c(fact, 'f') && ge_has_nan(layout, n, n, af, ldaf)) return -8;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -14;
    if (lsame_c(fact, 'f') && (lsame_c(*equed, 'b') || lsame_c(*equed, 'c')) && vec_has_nan(n, c)) return -13;
    if (lsame_c(fact, 'f') && (lsame_c(*equed, 'b') || lsame_c(*equed, 'r')) && vec_has_nan(n, r)) return -12;
  }
  lapack_int* iwork = alloc<lapack_int>((size_t)std::max(1, n));
  double* work = iwork ? alloc<double>((size_t)std::max(1, 4 * n)) : nullptr;
  if (!work) {
    if (iwork) LAPACKE_free_proxy(iwork);
    LAPACKE_xerbla("LAPACKE_dgesvx", LAPACK_WORK_MEMORY_ERROR);
    return LAPACK_WORK_MEMORY_ERROR;
  }
  lapack_int info = LAPACKE_dgesvx_work(layout, fact, trans, n, nrhs, a, lda, af, ldaf, ipiv, equed, r, c, b, ldb, x,
                                        ldx, rcond, ferr, berr, work, iwork);
  *rpivot = work[0];
  LAPACKE_free_proxy(work);
  LAPACKE_free_proxy(iwork);
  return info;
}

// ---------------------------------------------------------------- GETRI
// LAPACKE/src/lapacke_dgetri.c, lapacke_dgetri_work.c: NaN check of A (-3);
// the workspace is sized by a query; row major: LDA < N gives -4, the query
// passes LDA_T, A is transposed in and out.
lapack_int LAPACKE_dgetri_work(int layout, lapack_int n, double* a, lapack_int lda, const lapack_int* ipiv,
                               double* work, lapack_int lwork) {
  lapack_int info = 0;
  const char* nm = "LAPACKE_dgetri_work";
  if (layout == LAPACK_COL_MAJOR) {
    dgetri_(&n, a, &lda, ipiv, work, &lwork, &info);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -4); return -4; }
  if (lwork == -1) {
    dgetri_(&n, a, &lda_t, ipiv, work, &lwork, &info);
    return (info < 0) ? (info - 1) : info;
  }
  double* a_t = alloc<double>((size_t)lda_t * std::max(1, n));
  if (!a_t) { LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR); return LAPACK_TRANSPOSE_MEMORY_ERROR; }
  ge_trans(layout, n, n, a, lda, a_t, lda_t);
  dgetri_(&n, a_t, &lda_t, ipiv, work, &lwork, &info);
  if (info < 0) info -= 1;
  ge_trans(LAPACK_COL_MAJOR, n, n, a_t, lda_t, a, lda);
  LAPACKE_free_proxy(a_t);
  return info;
}
lapack_int LAPACKE_dgetri(int layout, lapack_int n, double* a, lapack_int lda, const lapack_int* ipiv) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dgetri", -1); return -1; }
  if (nancheck() && ge_has_nan(layout, n, n, a, lda)) return -3;
  double query = 0.0;
  lapack_int info = LAPACKE_dgetri_work(layout, n, a, lda, ipiv, &query, -1);
  if (info != 0) return info;
  const lapack_int lwork = (lapack_int)query;
  double* work = static_cast<double*>(LAPACKE_malloc_proxy(sizeof(double) * (size_t)lwork));
  if (!work) {
    LAPACKE_xerbla("LAPACKE_dgetri", LAPACK_WORK_MEMORY_ERROR);
    return LAPACK_WORK_MEMORY_ERROR;
  }
  info = LAPACKE_dgetri_work(layout, n, a, lda, ipiv, work, lwork);
  LAPACKE_free_proxy(work);
  return info;
}

// ---------------------------------------------------------------- POTRF / POTRS / POSV / SPOSV
lapack_int LAPACKE_dpotrf_work(int layout, char uplo, lapack_int n, double* a, lapack_int lda) {
  return potrf_work<double>("LAPACKE_dpotrf_work", dpotrf_, layout, uplo, n, a, lda);
}
lapack_int LAPACKE_spotrf_work(int layout, char uplo, lapack_int n, float* a, lapack_int lda) {
  return potrf_work<float>("LAPACKE_spotrf_work", spotrf_, layout, uplo, n, a, lda);
}
lapack_int LAPACKE_dpotrf(int layout, char uplo, lapack_int n, double* a, lapack_int lda) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dpotrf", -1); return -1; }
  if (nancheck() && tr_has_nan(layout, uplo, n, a, lda)) return -4;
  return LAPACKE_dpotrf_work(layout, uplo, n, a, lda);
}
lapack_int LAPACKE_spotrf(int layout, char uplo, lapack_int n, float* a, lapack_int lda) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_spotrf", -1); return -1; }
  if (nancheck() && tr_has_nan(layout, uplo, n, a, lda)) return -4;
  return LAPACKE_spotrf_work(layout, uplo, n, a, lda);
}
lapack_int LAPACKE_dpotrs_work(int layout, char uplo, lapack_int n, lapack_int nrhs, const double* a, lapack_int lda,
                               double* b, lapack_int ldb) {
  return potrs_posv_work<double>("LAPACKE_dpotrs_work",
                                 [](const char* u, const lapack_int* nn, const lapack_int* nr, double* aa,
                                    const lapack_int* la, double* bb, const lapack_int* lb, lapack_int* inf,
                                    size_t len) { dpotrs_(u, nn, nr, aa, la, bb, lb, inf, len); },
                                 false, layout, uplo, n, nrhs, const_cast<double*>(a), lda, b, ldb);
}
lapack_int LAPACKE_spotrs_work(int layout, char uplo, lapack_int n, lapack_int nrhs, const float* a, lapack_int lda,
                               float* b, lapack_int ldb) {
  return potrs_posv_work<float>("LAPACKE_spotrs_work",
                                [](const char* u, const lapack_int* nn, const lapack_int* nr, float* aa,
                                   const lapack_int* la, float* bb, const lapack_int* lb, lapack_int* inf,
                                   size_t len) { spotrs_(u, nn, nr, aa, la, bb, lb, inf, len); },
                                false, layout, uplo, n, nrhs, const_cast<float*>(a), lda, b, ldb);
}
lapack_int LAPACKE_dpotrs(int layout, char uplo, lapack_int n, lapack_int nrhs, const double* a, lapack_int lda,
                          double* b, lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dpotrs", -1); return -1; }
  if (nancheck()) {
    if (tr_has_nan(layout, uplo, n, a, lda)) return -5;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -7;
  }
  return LAPACKE_dpotrs_work(layout, uplo, n, nrhs, a, lda, b, ldb);
}
lapack_int LAPACKE_spotrs(int layout, char uplo, lapack_int n, lapack_int nrhs, const float* a, lapack_int lda,
                          float* b, lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_spotrs", -1); return -1; }
  if (nancheck()) {
    if (tr_has_nan(layout, uplo, n, a, lda)) return -5;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -7;
  }
  return LAPACKE_spotrs_work(layout, uplo, n, nrhs, a, lda, b, ldb);
}
lapack_int LAPACKE_dposv_work(int layout, char uplo, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                              double* b, lapack_int ldb) {
  return potrs_posv_work<double>("LAPACKE_dposv_work", dposv_, true, layout, uplo, n, nrhs, a, lda, b, ldb);
}
lapack_int LAPACKE_dposv(int layout, char uplo, lapack_int n, lapack_int nrhs, double* a, lapack_int lda, double* b,
                         lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dposv", -1); return -1; }
  if (nancheck()) {
    if (tr_has_nan(layout, uplo, n, a, lda)) return -5;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -7;
  }
  return LAPACKE_dposv_work(layout, uplo, n, nrhs, a, lda, b, ldb);
}
lapack_int LAPACKE_dsposv_work(int layout, char uplo, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                               const double* b, lapack_int ldb, double* x, lapack_int ldx, double* work, float* swork,
                               lapack_int* iter) {
  // LAPACKE/src/lapacke_dsposv_work.c: row major LDA < N -6, LDB < NRHS -8,
  // LDX < NRHS -10; A (the triangle) and X written back
  lapack_int info = 0;
  const char* nm = "LAPACKE_dsposv_work";
  if (layout == LAPACK_COL_MAJOR) {
    dsposv_(&uplo, &n, &nrhs, a, &lda, b, &ldb, x, &ldx, work, swork, iter, &info, 1);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n), ldb_t = std::max(1, n), ldx_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -6); return -6; }
  if (ldb < nrhs) { LAPACKE_xerbla(nm, -8); return -8; }
  if (ldx < nrhs) { LAPACKE_xerbla(nm, -10); return -10; }
  double* a_t = alloc<double>((size_t)lda_t * std::max(1, n));
  double* b_t = a_t ? alloc<double>((size_t)ldb_t * std::max(1, nrhs)) : nullptr;
  double* x_t = b_t ? alloc<double>((size_t)ldx_t * std::max(1, nrhs)) : nullptr;
  if (!x_t) {
    if (b_t) LAPACKE_free_proxy(b_t);
    if (a_t) LAPACKE_free_proxy(a_t);
    LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR);
    return LAPACK_TRANSPOSE_MEMORY_ERROR;
  }
  tr_trans(layout, uplo, n, a, lda, a_t, lda_t);
  ge_trans(layout, n, nrhs, b, ldb, b_t, ldb_t);
  dsposv_(&uplo, &n, &nrhs, a_t, &lda_t, b_t, &ldb_t, x_t, &ldx_t, work, swork, iter, &info, 1);
  if (info < 0) info -= 1;
  tr_trans(LAPACK_COL_MAJOR, uplo, n, a_t, lda_t, a, lda);
  ge_trans(LAPACK_COL_MAJOR, n, nrhs, x_t, ldx_t, x, ldx);
  LAPACKE_free_proxy(x_t);
  LAPACKE_free_proxy(b_t);
  LAPACKE_free_proxy(a_t);
  return info;
}
lapack_int LAPACKE_dsposv(int layout, char uplo, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                          const double* b, lapack_int ldb, double* x, lapack_int ldx, lapack_int* iter) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_dsposv", -1); return -1; }
  if (nancheck()) {
    if (tr_has_nan(layout, uplo, n, a, lda)) return -5;
    if (ge_has_nan(layout, n, nrhs, b, ldb)) return -7;
  }
  float* swork = alloc<float>((size_t)std::max(1, n) * std::max(1, n + nrhs));
  double* work = swork ? alloc<double>((size_t)std::max(1, n) * std::max(1, nrhs)) : nullptr;
  if (!work) {
    if (swork) LAPACKE_free_proxy(swork);
    LAPACKE_xerbla("LAPACKE_dsposv", LAPACK_WORK_MEMORY_ERROR);
    return LAPACK_WORK_MEMORY_ERROR;
  }
  lapack_int info = LAPACKE_dsposv_work(layout, uplo, n, nrhs, a, lda, b, ldb, x, ldx, work, swork, iter);
  LAPACKE_free_proxy(work);
  LAPACKE_free_proxy(swork);
  return info;
}


// ---------------------------------------------------------------- complex LU
// LAPACKE/src/lapacke_{z,c}getrf*.c, {z,c}getrs*.c, {z,c}gesv*.c, zcgesv*.c
lapack_int LAPACKE_zgetrf_work(int layout, lapack_int m, lapack_int n, void* a, lapack_int lda, lapack_int* ipiv) {
  return getrf_work<zc_t>("LAPACKE_zgetrf_work", zgetrf_, layout, m, n, static_cast<zc_t*>(a), lda, ipiv);
}
lapack_int LAPACKE_cgetrf_work(int layout, lapack_int m, lapack_int n, void* a, lapack_int lda, lapack_int* ipiv) {
  return getrf_work<cc_t>("LAPACKE_cgetrf_work", cgetrf_, layout, m, n, static_cast<cc_t*>(a), lda, ipiv);
}
lapack_int LAPACKE_zgetrf(int layout, lapack_int m, lapack_int n, void* a, lapack_int lda, lapack_int* ipiv) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_zgetrf", -1); return -1; }
  if (nancheck() && ge_has_nan(layout, m, n, static_cast<const zc_t*>(a), lda)) return -4;
  return LAPACKE_zgetrf_work(layout, m, n, a, lda, ipiv);
}
lapack_int LAPACKE_cgetrf(int layout, lapack_int m, lapack_int n, void* a, lapack_int lda, lapack_int* ipiv) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_cgetrf", -1); return -1; }
  if (nancheck() && ge_has_nan(layout, m, n, static_cast<const cc_t*>(a), lda)) return -4;
  return LAPACKE_cgetrf_work(layout, m, n, a, lda, ipiv);
}
lapack_int LAPACKE_zgetrs_work(int layout, char trans, lapack_int n, lapack_int nrhs, const void* a, lapack_int lda,
                               const lapack_int* ipiv, void* b, lapack_int ldb) {
  return getrs_work<zc_t>("LAPACKE_zgetrs_work", zgetrs_, layout, trans, n, nrhs, static_cast<const zc_t*>(a), lda,
                          ipiv, static_cast<zc_t*>(b), ldb);
}
lapack_int LAPACKE_cgetrs_work(int layout, char trans, lapack_int n, lapack_int nrhs, const void* a, lapack_int lda,
                               const lapack_int* ipiv, void* b, lapack_int ldb) {
  return getrs_work<cc_t>("LAPACKE_cgetrs_work", cgetrs_, layout, trans, n, nrhs, static_cast<const cc_t*>(a), lda,
                          ipiv, static_cast<cc_t*>(b), ldb);
}
lapack_int LAPACKE_zgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const void* a, lapack_int lda,
                          const lapack_int* ipiv, void* b, lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_zgetrs", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, static_cast<const zc_t*>(a), lda)) return -5;
    if (ge_has_nan(layout, n, nrhs, static_cast<const zc_t*>(b), ldb)) return -8;
  }
  return LAPACKE_zgetrs_work(layout, trans, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_cgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const void* a, lapack_int lda,
                          const lapack_int* ipiv, void* b, lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_cgetrs", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, static_cast<const cc_t*>(a), lda)) return -5;
    if (ge_has_nan(layout, n, nrhs, static_cast<const cc_t*>(b), ldb)) return -8;
  }
  return LAPACKE_cgetrs_work(layout, trans, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_zgesv_work(int layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda, lapack_int* ipiv,
                              void* b, lapack_int ldb) {
  return gesv_work<zc_t>("LAPACKE_zgesv_work", zgesv_, layout, n, nrhs, static_cast<zc_t*>(a), lda, ipiv,
                         static_cast<zc_t*>(b), ldb);
}
lapack_int LAPACKE_cgesv_work(int layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda, lapack_int* ipiv,
                              void* b, lapack_int ldb) {
  return gesv_work<cc_t>("LAPACKE_cgesv_work", cgesv_, layout, n, nrhs, static_cast<cc_t*>(a), lda, ipiv,
                         static_cast<cc_t*>(b), ldb);
}
lapack_int LAPACKE_zgesv(int layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda, lapack_int* ipiv, void* b,
                         lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_zgesv", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, static_cast<const zc_t*>(a), lda)) return -4;
    if (ge_has_nan(layout, n, nrhs, static_cast<const zc_t*>(b), ldb)) return -7;
  }
  return LAPACKE_zgesv_work(layout, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_cgesv(int layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda, lapack_int* ipiv, void* b,
                         lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_cgesv", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, static_cast<const cc_t*>(a), lda)) return -4;
    if (ge_has_nan(layout, n, nrhs, static_cast<const cc_t*>(b), ldb)) return -7;
  }
  return LAPACKE_cgesv_work(layout, n, nrhs, a, lda, ipiv, b, ldb);
}
lapack_int LAPACKE_zcgesv_work(int layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda, lapack_int* ipiv,
                               const void* b, lapack_int ldb, void* x, lapack_int ldx, void* work, void* swork,
                               double* rwork, lapack_int* iter) {
  // LAPACKE/src/lapacke_zcgesv_work.c: row major LDA < N -5, LDB < NRHS -8,
  // LDX < NRHS -10; A and X written back
  lapack_int info = 0;
  const char* nm = "LAPACKE_zcgesv_work";
  if (layout == LAPACK_COL_MAJOR) {
    zcgesv_(&n, &nrhs, a, &lda, ipiv, b, &ldb, x, &ldx, work, swork, rwork, iter, &info);
    if (info < 0) info -= 1;
    return info;
  }
  if (layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla(nm, -1); return -1; }
  lapack_int lda_t = std::max(1, n), ldb_t = std::max(1, n), ldx_t = std::max(1, n);
  if (lda < n) { LAPACKE_xerbla(nm, -5); return -5; }
  if (ldb < nrhs) { LAPACKE_xerbla(nm, -8); return -8; }
  if (ldx < nrhs) { LAPACKE_xerbla(nm, -10); return -10; }
  zc_t* a_t = alloc<zc_t>((size_t)lda_t * std::max(1, n));
  zc_t* b_t = a_t ? alloc<zc_t>((size_t)ldb_t * std::max(1, nrhs)) : nullptr;
  zc_t* x_t = b_t ? alloc<zc_t>((size_t)ldx_t * std::max(1, nrhs)) : nullptr;
  if (!x_t) {
    if (b_t) LAPACKE_free_proxy(b_t);
    if (a_t) LAPACKE_free_proxy(a_t);
    LAPACKE_xerbla(nm, LAPACK_TRANSPOSE_MEMORY_ERROR);
    return LAPACK_TRANSPOSE_MEMORY_ERROR;
  }
  ge_trans(layout, n, n, static_cast<const zc_t*>(a), lda, a_t, lda_t);
  ge_trans(layout, n, nrhs, static_cast<const zc_t*>(b), ldb, b_t, ldb_t);
  zcgesv_(&n, &nrhs, a_t, &lda_t, ipiv, b_t, &ldb_t, x_t, &ldx_t, work, swork, rwork, iter, &info);
  if (info < 0) info -= 1;
  ge_trans(LAPACK_COL_MAJOR, n, n, a_t, lda_t, static_cast<zc_t*>(a), lda);
  ge_trans(LAPACK_COL_MAJOR, n, nrhs, x_t, ldx_t, static_cast<zc_t*>(x), ldx);
  LAPACKE_free_proxy(x_t);
  LAPACKE_free_proxy(b_t);
  LAPACKE_free_proxy(a_t);
  return info;
}
lapack_int LAPACKE_zcgesv(int layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda, lapack_int* ipiv,
                          const void* b, lapack_int ldb, void* x, lapack_int ldx, lapack_int* iter) {
  if (layout != LAPACK_COL_MAJOR && layout != LAPACK_ROW_MAJOR) { LAPACKE_xerbla("LAPACKE_zcgesv", -1); return -1; }
  if (nancheck()) {
    if (ge_has_nan(layout, n, n, static_cast<const zc_t*>(a), lda)) return -4;
    if (ge_has_nan(layout, n, nrhs, static_cast<const zc_t*>(b), ldb)) return -7;
  }
  // RWORK, SWORK, WORK as LAPACKE_zcgesv allocates them
  double* rwork = alloc<double>((size_t)std::max(1, n));
  cc_t* swork = rwork ? alloc<cc_t>((size_t)std::max(1, n) * std::max(1, n + nrhs)) : nullptr;
  zc_t* work = swork ? alloc<zc_t>((size_t)std::max(1, n) * std::max(1, nrhs)) : nullptr;
  if (!work) {
    if (swork) LAPACKE_free_proxy(swork);
    if (rwork) LAPACKE_free_proxy(rwork);
    LAPACKE_xerbla("LAPACKE_zcgesv", LAPACK_WORK_MEMORY_ERROR);
    return LAPACK_WORK_MEMORY_ERROR;
  }
  lapack_int info = LAPACKE_zcgesv_work(layout, n, nrhs, a, lda, ipiv, b, ldb, x, ldx, work, swork, rwork, iter);
  LAPACKE_free_proxy(work);
  LAPACKE_free_proxy(swork);
  LAPACKE_free_proxy(rwork);
  return info;
}

}  // extern "C"
