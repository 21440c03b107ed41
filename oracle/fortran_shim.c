/*
 * ORACLE test infrastructure: Fortran-ABI entry points (dgesv_, dgetrf_, ...)
 * over the C restatement, so that the reference's own LAPACKE C wrappers can
 * be compiled from the reference sources and run on top of the oracle.
 * Argument lists follow LAPACKE/include/lapack.h (hidden CHARACTER lengths
 * at the end, LAPACK_FORTRAN_STRLEN_END).  Linked only into _ref/.
 */
#include <stddef.h>
void or_dgesv(int, int, double *, int, int *, double *, int, int *);
void or_sgesv(int, int, float *, int, int *, float *, int, int *);
void or_dgetrf(int, int, double *, int, int *, int *);
void or_sgetrf(int, int, float *, int, int *, int *);
void or_dgetrf2(int, int, double *, int, int *, int *);
void or_sgetrf2(int, int, float *, int, int *, int *);
void or_dgetrs(char, int, int, const double *, int, const int *, double *, int, int *);
void or_sgetrs(char, int, int, const float *, int, const int *, float *, int, int *);
void or_dlaswp(int, double *, int, int, int, const int *, int);
void or_slaswp(int, float *, int, int, int, const int *, int);
void or_dlag2s(int, int, const double *, int, float *, int, int *);
void or_slag2d(int, int, const float *, int, double *, int, int *);
void or_dsgesv(int, int, double *, int, int *, const double *, int, double *, int, double *, float *, int *, int *);
void or_dgecon(char, int, const double *, int, double, double *, double *, int *, int *);
void or_dgetri(int, double *, int, const int *, double *, int, int, int *);
void or_dpotrf(char, int, double *, int, int *);
void or_spotrf(char, int, float *, int, int *);
void or_dpotrs(char, int, int, const double *, int, double *, int, int *);
void or_spotrs(char, int, int, const float *, int, float *, int, int *);
void or_dposv(char, int, int, double *, int, double *, int, int *);
void or_dsposv(char, int, int, double *, int, const double *, int, double *, int, double *, float *, int *, int *);
void or_dgerfs(char, int, int, const double *, int, const double *, int, const int *, const double *, int, double *,
               int, double *, double *, double *, int *, int *);
void or_dgesvx(char, char, int, int, double *, int, double *, int, int *, char *, double *, double *, double *, int,
               double *, int, double *, double *, double *, double *, int *, int *);

void dgesv_(const int *n, const int *nrhs, double *a, const int *lda, int *ipiv, double *b, const int *ldb, int *info) {
  or_dgesv(*n, *nrhs, a, *lda, ipiv, b, *ldb, info);
}
void sgesv_(const int *n, const int *nrhs, float *a, const int *lda, int *ipiv, float *b, const int *ldb, int *info) {
  or_sgesv(*n, *nrhs, a, *lda, ipiv, b, *ldb, info);
}
void dgetrf_(const int *m, const int *n, double *a, const int *lda, int *ipiv, int *info) {
  or_dgetrf(*m, *n, a, *lda, ipiv, info);
}
void sgetrf_(const int *m, const int *n, float *a, const int *lda, int *ipiv, int *info) {
  or_sgetrf(*m, *n, a, *lda, ipiv, info);
}
void dgetrf2_(const int *m, const int *n, double *a, const int *lda, int *ipiv, int *info) {
  or_dgetrf2(*m, *n, a, *lda, ipiv, info);
}
void sgetrf2_(const int *m, const int *n, float *a, const int *lda, int *ipiv, int *info) {
  or_sgetrf2(*m, *n, a, *lda, ipiv, info);
}
void dgetrs_(const char *trans, const int *n, const int *nrhs, const double *a, const int *lda, const int *ipiv,
             double *b, const int *ldb, int *info, size_t trans_len) {
  (void)trans_len;
  or_dgetrs(*trans, *n, *nrhs, a, *lda, ipiv, b, *ldb, info);
}
void sgetrs_(const char *trans, const int *n, const int *nrhs, const float *a, const int *lda, const int *ipiv,
             float *b, const int *ldb, int *info, size_t trans_len) {
  (void)trans_len;
  or_sgetrs(*trans, *n, *nrhs, a, *lda, ipiv, b, *ldb, info);
}
void dlaswp_(const int *n, double *a, const int *lda, const int *k1, const int *k2, const int *ipiv, const int *incx) {
  or_dlaswp(*n, a, *lda, *k1, *k2, ipiv, *incx);
}
void slaswp_(const int *n, float *a, const int *lda, const int *k1, const int *k2, const int *ipiv, const int *incx) {
  or_slaswp(*n, a, *lda, *k1, *k2, ipiv, *incx);
}
void dlag2s_(const int *m, const int *n, const double *a, const int *lda, float *sa, const int *ldsa, int *info) {
  or_dlag2s(*m, *n, a, *lda, sa, *ldsa, info);
}
void slag2d_(const int *m, const int *n, const float *sa, const int *ldsa, double *a, const int *lda, int *info) {
  or_slag2d(*m, *n, sa, *ldsa, a, *lda, info);
}
void dsgesv_(const int *n, const int *nrhs, double *a, const int *lda, int *ipiv, const double *b, const int *ldb,
             double *x, const int *ldx, double *work, float *swork, int *iter, int *info) {
  or_dsgesv(*n, *nrhs, a, *lda, ipiv, b, *ldb, x, *ldx, work, swork, iter, info);
}
void dgecon_(const char *norm, const int *n, const double *a, const int *lda, const double *anorm, double *rcond,
             double *work, int *iwork, int *info, size_t norm_len) {
  (void)norm_len;
  or_dgecon(*norm, *n, a, *lda, *anorm, rcond, work, iwork, info);
}
void dgerfs_(const char *trans, const int *n, const int *nrhs, const double *a, const int *lda, const double *af,
             const int *ldaf, const int *ipiv, const double *b, const int *ldb, double *x, const int *ldx,
             double *ferr, double *berr, double *work, int *iwork, int *info, size_t trans_len) {
  (void)trans_len;
  or_dgerfs(*trans, *n, *nrhs, a, *lda, af, *ldaf, ipiv, b, *ldb, x, *ldx, ferr, berr, work, iwork, info);
}
void dgesvx_(const char *fact, const char *trans, const int *n, const int *nrhs, double *a, const int *lda,
             double *af, const int *ldaf, int *ipiv, char *equed, double *r, double *c, double *b, const int *ldb,
             double *x, const int *ldx, double *rcond, double *ferr, double *berr, double *work, int *iwork,
             int *info, size_t fact_len, size_t trans_len, size_t equed_len) {
  (void)fact_len;
  (void)trans_len;
  (void)equed_len;
  or_dgesvx(*fact, *trans, *n, *nrhs, a, *lda, af, *ldaf, ipiv, equed, r, c, b, *ldb, x, *ldx, rcond, ferr, berr,
            work, iwork, info);
}
void dgetri_(const int *n, double *a, const int *lda, const int *ipiv, double *work, const int *lwork, int *info) {
  or_dgetri(*n, a, *lda, ipiv, work, *lwork, 64, info);   /* NB = ILAENV(1, 'DGETRI') = 64 */
}
void dpotrf_(const char *uplo, const int *n, double *a, const int *lda, int *info, size_t l) {
  (void)l;
  or_dpotrf(*uplo, *n, a, *lda, info);
}
void spotrf_(const char *uplo, const int *n, float *a, const int *lda, int *info, size_t l) {
  (void)l;
  or_spotrf(*uplo, *n, a, *lda, info);
}
void dpotrs_(const char *uplo, const int *n, const int *nrhs, const double *a, const int *lda, double *b,
             const int *ldb, int *info, size_t l) {
  (void)l;
  or_dpotrs(*uplo, *n, *nrhs, a, *lda, b, *ldb, info);
}
void spotrs_(const char *uplo, const int *n, const int *nrhs, const float *a, const int *lda, float *b,
             const int *ldb, int *info, size_t l) {
  (void)l;
  or_spotrs(*uplo, *n, *nrhs, a, *lda, b, *ldb, info);
}
void dposv_(const char *uplo, const int *n, const int *nrhs, double *a, const int *lda, double *b, const int *ldb,
            int *info, size_t l) {
  (void)l;
  or_dposv(*uplo, *n, *nrhs, a, *lda, b, *ldb, info);
}
void dsposv_(const char *uplo, const int *n, const int *nrhs, double *a, const int *lda, const double *b,
             const int *ldb, double *x, const int *ldx, double *work, float *swork, int *iter, int *info, size_t l) {
  (void)l;
  or_dsposv(*uplo, *n, *nrhs, a, *lda, b, *ldb, x, *ldx, work, swork, iter, info);
}

void or_zgetrf(int, int, void *, int, int *, int *);
void or_zgetrs(char, int, int, const void *, int, const int *, void *, int, int *);
void or_zgesv(int, int, void *, int, int *, void *, int, int *);
void zgetrf_(const int *m, const int *n, void *a, const int *lda, int *ipiv, int *info) {
  or_zgetrf(*m, *n, a, *lda, ipiv, info);
}
void zgetrs_(const char *trans, const int *n, const int *nrhs, const void *a, const int *lda, const int *ipiv,
             void *b, const int *ldb, int *info, size_t l) {
  (void)l;
  or_zgetrs(*trans, *n, *nrhs, a, *lda, ipiv, b, *ldb, info);
}
void zgesv_(const int *n, const int *nrhs, void *a, const int *lda, int *ipiv, void *b, const int *ldb, int *info) {
  or_zgesv(*n, *nrhs, a, *lda, ipiv, b, *ldb, info);
}
void or_cgetrf(int, int, void *, int, int *, int *);
void or_cgetrs(char, int, int, const void *, int, const int *, void *, int, int *);
void or_cgesv(int, int, void *, int, int *, void *, int, int *);
void or_zcgesv(int, int, void *, int, int *, const void *, int, void *, int, void *, void *, double *, int *, int *);
void cgetrf_(const int *m, const int *n, void *a, const int *lda, int *ipiv, int *info) {
  or_cgetrf(*m, *n, a, *lda, ipiv, info);
}
void or_zgetrf2(int, int, void *, int, int *, int *);
void or_cgetrf2(int, int, void *, int, int *, int *);
void zgetrf2_(const int *m, const int *n, void *a, const int *lda, int *ipiv, int *info) {
  or_zgetrf2(*m, *n, a, *lda, ipiv, info);
}
void cgetrf2_(const int *m, const int *n, void *a, const int *lda, int *ipiv, int *info) {
  or_cgetrf2(*m, *n, a, *lda, ipiv, info);
}
void cgetrs_(const char *trans, const int *n, const int *nrhs, const void *a, const int *lda, const int *ipiv,
             void *b, const int *ldb, int *info, size_t l) {
  (void)l;
  or_cgetrs(*trans, *n, *nrhs, a, *lda, ipiv, b, *ldb, info);
}
void cgesv_(const int *n, const int *nrhs, void *a, const int *lda, int *ipiv, void *b, const int *ldb, int *info) {
  or_cgesv(*n, *nrhs, a, *lda, ipiv, b, *ldb, info);
}
void zcgesv_(const int *n, const int *nrhs, void *a, const int *lda, int *ipiv, const void *b, const int *ldb,
             void *x, const int *ldx, void *work, void *swork, double *rwork, int *iter, int *info) {
  or_zcgesv(*n, *nrhs, a, *lda, ipiv, b, *ldb, x, *ldx, work, swork, rwork, iter, info);
}

/* LSAME (INSTALL/lsame.f): case-insensitive comparison of one character. */
int lsame_(const char *ca, const char *cb, size_t la, size_t lb) {
  (void)la;
  (void)lb;
  char a = *ca, b = *cb;
  if (a >= 'a' && a <= 'z') a = (char)(a - 32);
  if (b >= 'a' && b <= 'z') b = (char)(b - 32);
  return a == b;
}
