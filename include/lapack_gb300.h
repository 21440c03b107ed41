/*
 * lapack_gb300.h -- C ABI of the GB300 dense LU solve library.
 *
 * Three layers, all plain C types (no CUDA or torch types in signatures;
 * a stream is passed as void*):
 *
 *  1. The LAPACK Fortran ABI for the LU solve path, so an existing Fortran
 *     or C program links against liblapack_gb300.so in place of the
 *     reference LAPACK for these routines.  Host pointers, column-major,
 *     1-based IPIV, INFO as in the reference; the library copies to the GPU
 *     and back inside each call and retains no pointer.  Hidden CHARACTER
 *     lengths come last (LAPACK_FORTRAN_STRLEN_END convention).
 *  2. The LAPACKE C interface for the same routines (row/column major,
 *     NaN checks, INFO shifts, LAPACKE_NANCHECK).
 *  3. gb300_* device-pointer entry points for callers whose data already
 *     lives in GPU memory (no reference counterpart), plus option and
 *     status controls.
 *
 * lapack_int is 32-bit (LP64), matching the reference default.
 */
#ifndef LAPACK_GB300_H
#define LAPACK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t lapack_int;

/* ---------------------------------------------------------------------
 * 1. Fortran ABI (LAPACKE/include/lapack.h prototypes)
 * ------------------------------------------------------------------- */

/* LU with partial pivoting, blocked right-looking.
 * Replaces SRC/dgetrf.f:105 (prototype LAPACKE/include/lapack.h:4349-4355). */
void dgetrf_(const lapack_int* m, const lapack_int* n, double* a, const lapack_int* lda,
             lapack_int* ipiv, lapack_int* info);
/* Replaces SRC/sgetrf.f (lapack.h:4363-4369). */
void sgetrf_(const lapack_int* m, const lapack_int* n, float* a, const lapack_int* lda,
             lapack_int* ipiv, lapack_int* info);
/* Recursive panel LU.  Replaces SRC/dgetrf2.f:112 (lapack.h:4373-4379). */
void dgetrf2_(const lapack_int* m, const lapack_int* n, double* a, const lapack_int* lda,
              lapack_int* ipiv, lapack_int* info);
/* Replaces SRC/sgetrf2.f (lapack.h:4387-4393). */
void sgetrf2_(const lapack_int* m, const lapack_int* n, float* a, const lapack_int* lda,
              lapack_int* ipiv, lapack_int* info);
/* Solve with the LU factors, TRANS = 'N', 'T' or 'C'.
 * Replaces SRC/dgetrs.f:118 (lapack.h:4436-4451). */
void dgetrs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const double* a,
             const lapack_int* lda, const lapack_int* ipiv, double* b, const lapack_int* ldb,
             lapack_int* info, size_t trans_len);
/* Replaces SRC/sgetrs.f (lapack.h:4453-4468). */
void sgetrs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const float* a,
             const lapack_int* lda, const lapack_int* ipiv, float* b, const lapack_int* ldb,
             lapack_int* info, size_t trans_len);
/* Driver: DGETRF then DGETRS('N').  Replaces SRC/dgesv.f:121 (lapack.h:3706-3712). */
void dgesv_(const lapack_int* n, const lapack_int* nrhs, double* a, const lapack_int* lda,
            lapack_int* ipiv, double* b, const lapack_int* ldb, lapack_int* info);
/* Replaces SRC/sgesv.f (lapack.h sgesv prototype). */
void sgesv_(const lapack_int* n, const lapack_int* nrhs, float* a, const lapack_int* lda,
            lapack_int* ipiv, float* b, const lapack_int* ldb, lapack_int* info);
/* Mixed-precision iterative refinement driver.
 * Replaces SRC/dsgesv.f:191 (lapack.h:3727-3735).  WORK and SWORK are
 * accepted for ABI compatibility; the computation uses device memory. */
void dsgesv_(const lapack_int* n, const lapack_int* nrhs, double* a, const lapack_int* lda,
             lapack_int* ipiv, const double* b, const lapack_int* ldb, double* x,
             const lapack_int* ldx, double* work, float* swork, lapack_int* iter, lapack_int* info);
/* Iterative refinement with error bounds.  Replaces SRC/dgerfs.f:181
 * (lapack.h:3158-3174).  X is refined in place with the factors AF/IPIV of
 * A (from DGETRF); FERR/BERR receive the forward error bound and the
 * componentwise backward error of each column.  WORK (3N) and IWORK (N) are
 * accepted and unused: the vectors live in GPU memory. */
void dgerfs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const double* a,
             const lapack_int* lda, const double* af, const lapack_int* ldaf, const lapack_int* ipiv,
             const double* b, const lapack_int* ldb, double* x, const lapack_int* ldx, double* ferr,
             double* berr, double* work, lapack_int* iwork, lapack_int* info, size_t trans_len);
/* Reciprocal condition number from the LU factors.  Replaces SRC/dgecon.f:124
 * (lapack.h:1513-1526).  WORK (4N) and IWORK (N) are accepted and unused. */
void dgecon_(const char* norm, const lapack_int* n, const double* a, const lapack_int* lda,
             const double* anorm, double* rcond, double* work, lapack_int* iwork, lapack_int* info,
             size_t norm_len);
/* Triangular solve with overflow protection, op(A) x = s*b.  Replaces
 * SRC/dlatrs.f:238 (the auxiliary routine DGECON calls).  CNORM is input
 * when NORMIN = 'Y', else output; SCALE receives s. */
void dlatrs_(const char* uplo, const char* trans, const char* diag, const char* normin, const lapack_int* n,
             const double* a, const lapack_int* lda, double* x, double* scale, double* cnorm, lapack_int* info,
             size_t uplo_len, size_t trans_len, size_t diag_len, size_t normin_len);
/* Expert driver: optional equilibration, LU, condition estimate, solve,
 * refinement with error bounds.  Replaces SRC/dgesvx.f:344 (lapack.h:4118-4139).  WORK(1) receives the reciprocal pivot growth; IWORK
 * is accepted and unused. */
void dgesvx_(const char* fact, const char* trans, const lapack_int* n, const lapack_int* nrhs, double* a,
             const lapack_int* lda, double* af, const lapack_int* ldaf, lapack_int* ipiv, char* equed, double* r,
             double* c, double* b, const lapack_int* ldb, double* x, const lapack_int* ldx, double* rcond,
             double* ferr, double* berr, double* work, lapack_int* iwork, lapack_int* info, size_t fact_len,
             size_t trans_len, size_t equed_len);
/* Inverse from the LU factors.  Replaces SRC/dgetri.f:111
 * (lapack.h:4398-4404).  LWORK = -1 is the workspace query (WORK(1) = N*NB);
 * a smaller LWORK shrinks the block size as the reference does. */
void dgetri_(const lapack_int* n, double* a, const lapack_int* lda, const lapack_int* ipiv, double* work,
             const lapack_int* lwork, lapack_int* info);
/* Cholesky factorization, solve and driver of a symmetric positive
 * definite matrix (one triangle referenced).  Replace SRC/dpotrf.f:104,
 * SRC/spotrf.f, SRC/dpotrs.f:107, SRC/spotrs.f, SRC/dposv.f:127 (the
 * LAPACK_dpotrf, _spotrf, _dpotrs, _spotrs, _dposv prototypes of lapack.h). */
void dpotrf_(const char* uplo, const lapack_int* n, double* a, const lapack_int* lda, lapack_int* info,
             size_t uplo_len);
void spotrf_(const char* uplo, const lapack_int* n, float* a, const lapack_int* lda, lapack_int* info,
             size_t uplo_len);
void dpotrs_(const char* uplo, const lapack_int* n, const lapack_int* nrhs, const double* a, const lapack_int* lda,
             double* b, const lapack_int* ldb, lapack_int* info, size_t uplo_len);
void spotrs_(const char* uplo, const lapack_int* n, const lapack_int* nrhs, const float* a, const lapack_int* lda,
             float* b, const lapack_int* ldb, lapack_int* info, size_t uplo_len);
void dposv_(const char* uplo, const lapack_int* n, const lapack_int* nrhs, double* a, const lapack_int* lda,
            double* b, const lapack_int* ldb, lapack_int* info, size_t uplo_len);
/* Mixed-precision Cholesky refinement.  Replaces SRC/dsposv.f:195 (lapack.h
 * LAPACK_dsposv).  WORK and SWORK are accepted and unused. */
void dsposv_(const char* uplo, const lapack_int* n, const lapack_int* nrhs, double* a, const lapack_int* lda,
             const double* b, const lapack_int* ldb, double* x, const lapack_int* ldx, double* work, float* swork,
             lapack_int* iter, lapack_int* info, size_t uplo_len);
/* Complex LU factorization, solve and driver.  Replace SRC/zgetrf.f:105,
 * SRC/zgetrs.f:118 and SRC/zgesv.f:121 (the LAPACK_zgetrf, _zgetrs, _zgesv
 * prototypes of lapack.h).  COMPLEX*16 arrays are (re, im) pairs of doubles;
 * any lapack_complex_double* (C double _Complex, C++ std::complex<double>)
 * converts to the void* parameters. */
void zgetrf_(const lapack_int* m, const lapack_int* n, void* a, const lapack_int* lda, lapack_int* ipiv,
             lapack_int* info);
/* The recursive panel factorization alone.  Replaces SRC/zgetrf2.f:112 and
 * SRC/cgetrf2.f:112 (lapack.h LAPACK_zgetrf2, LAPACK_cgetrf2). */
void zgetrf2_(const lapack_int* m, const lapack_int* n, void* a, const lapack_int* lda, lapack_int* ipiv,
              lapack_int* info);
void cgetrf2_(const lapack_int* m, const lapack_int* n, void* a, const lapack_int* lda, lapack_int* ipiv,
              lapack_int* info);
void zgetrs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const void* a, const lapack_int* lda,
             const lapack_int* ipiv, void* b, const lapack_int* ldb, lapack_int* info, size_t trans_len);
void zgesv_(const lapack_int* n, const lapack_int* nrhs, void* a, const lapack_int* lda, lapack_int* ipiv, void* b,
            const lapack_int* ldb, lapack_int* info);
/* The COMPLEX twins.  Replace SRC/cgetrf.f:105, SRC/cgetrs.f:118,
 * SRC/cgesv.f:121 (lapack.h LAPACK_cgetrf, _cgetrs, _cgesv); arrays are
 * (re, im) pairs of floats. */
void cgetrf_(const lapack_int* m, const lapack_int* n, void* a, const lapack_int* lda, lapack_int* ipiv,
             lapack_int* info);
void cgetrs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const void* a, const lapack_int* lda,
             const lapack_int* ipiv, void* b, const lapack_int* ldb, lapack_int* info, size_t trans_len);
void cgesv_(const lapack_int* n, const lapack_int* nrhs, void* a, const lapack_int* lda, lapack_int* ipiv, void* b,
            const lapack_int* ldb, lapack_int* info);
/* Mixed-precision complex solve with refinement.  Replaces SRC/zcgesv.f:197
 * (lapack.h LAPACK_zcgesv).  WORK, SWORK and RWORK are accepted and unused. */
void zcgesv_(const lapack_int* n, const lapack_int* nrhs, void* a, const lapack_int* lda, lapack_int* ipiv,
             const void* b, const lapack_int* ldb, void* x, const lapack_int* ldx, void* work, void* swork,
             double* rwork, lapack_int* iter, lapack_int* info);
/* Row interchanges.  Replaces SRC/dlaswp.f:112 (lapack.h:11326-11332). */
void dlaswp_(const lapack_int* n, double* a, const lapack_int* lda, const lapack_int* k1,
             const lapack_int* k2, const lapack_int* ipiv, const lapack_int* incx);
/* Replaces SRC/slaswp.f (lapack.h slaswp prototype). */
void slaswp_(const lapack_int* n, float* a, const lapack_int* lda, const lapack_int* k1,
             const lapack_int* k2, const lapack_int* ipiv, const lapack_int* incx);
/* Precision conversions.  Replace SRC/dlag2s.f:105 and SRC/slag2d.f:101
 * (lapack.h:9748-9760). */
void dlag2s_(const lapack_int* m, const lapack_int* n, const double* a, const lapack_int* lda,
             float* sa, const lapack_int* ldsa, lapack_int* info);
void slag2d_(const lapack_int* m, const lapack_int* n, const float* sa, const lapack_int* ldsa,
             double* a, const lapack_int* lda, lapack_int* info);
/* Matrix norm, NORM = 'M', '1'/'O', 'I'.  Replaces SRC/dlange.f:111 for
 * those norms (lapack.h dlange prototype). */
double dlange_(const char* norm, const lapack_int* m, const lapack_int* n, const double* a,
               const lapack_int* lda, double* work, size_t norm_len);
/* Machine parameters.  Replace INSTALL/dlamch.f:68 and INSTALL/slamch.f. */
double dlamch_(const char* cmach, size_t len);
float slamch_(const char* cmach, size_t len);
/* Error handler.  Replaces SRC/xerbla.f:67: prints the reference message and
 * stops the program, unless gb300_xerbla_capture(1) is in effect.  Weak:
 * a program may supply its own xerbla_. */
void xerbla_(const char* srname, const lapack_int* info, size_t srname_len);

/* ---------------------------------------------------------------------
 * 2. LAPACKE (LAPACKE/include/lapacke.h)
 * ------------------------------------------------------------------- */
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
#define LAPACK_WORK_MEMORY_ERROR -1010
#define LAPACK_TRANSPOSE_MEMORY_ERROR -1011

/* LAPACKE/include/lapacke.h:939-952 */
lapack_int LAPACKE_dgesv(int matrix_layout, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                         lapack_int* ipiv, double* b, lapack_int ldb);
lapack_int LAPACKE_dgesv_work(int matrix_layout, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                              lapack_int* ipiv, double* b, lapack_int ldb);
lapack_int LAPACKE_sgesv(int matrix_layout, lapack_int n, lapack_int nrhs, float* a, lapack_int lda,
                         lapack_int* ipiv, float* b, lapack_int ldb);
lapack_int LAPACKE_sgesv_work(int matrix_layout, lapack_int n, lapack_int nrhs, float* a, lapack_int lda,
                              lapack_int* ipiv, float* b, lapack_int ldb);
/* LAPACKE/include/lapacke.h:1129-1167 */
lapack_int LAPACKE_dgetrf(int matrix_layout, lapack_int m, lapack_int n, double* a, lapack_int lda,
                          lapack_int* ipiv);
lapack_int LAPACKE_dgetrf_work(int matrix_layout, lapack_int m, lapack_int n, double* a, lapack_int lda,
                               lapack_int* ipiv);
lapack_int LAPACKE_dgetrf2(int matrix_layout, lapack_int m, lapack_int n, double* a, lapack_int lda,
                           lapack_int* ipiv);
lapack_int LAPACKE_dgetrf2_work(int matrix_layout, lapack_int m, lapack_int n, double* a, lapack_int lda,
                                lapack_int* ipiv);
lapack_int LAPACKE_sgetrf(int matrix_layout, lapack_int m, lapack_int n, float* a, lapack_int lda,
                          lapack_int* ipiv);
lapack_int LAPACKE_sgetrf_work(int matrix_layout, lapack_int m, lapack_int n, float* a, lapack_int lda,
                               lapack_int* ipiv);
lapack_int LAPACKE_dgetrs(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const double* a,
                          lapack_int lda, const lapack_int* ipiv, double* b, lapack_int ldb);
lapack_int LAPACKE_dgetrs_work(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const double* a,
                               lapack_int lda, const lapack_int* ipiv, double* b, lapack_int ldb);
lapack_int LAPACKE_sgetrs(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const float* a,
                          lapack_int lda, const lapack_int* ipiv, float* b, lapack_int ldb);
lapack_int LAPACKE_sgetrs_work(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const float* a,
                               lapack_int lda, const lapack_int* ipiv, float* b, lapack_int ldb);
/* LAPACKE/include/lapacke.h:2577 (dsgesv) */
lapack_int LAPACKE_dsgesv(int matrix_layout, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                          lapack_int* ipiv, const double* b, lapack_int ldb, double* x, lapack_int ldx,
                          lapack_int* iter);
lapack_int LAPACKE_dsgesv_work(int matrix_layout, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                               lapack_int* ipiv, const double* b, lapack_int ldb, double* x, lapack_int ldx,
                               double* work, float* swork, lapack_int* iter);
/* LAPACKE/include/lapacke.h (dlaswp, slaswp) */
lapack_int LAPACKE_dlaswp(int matrix_layout, lapack_int n, double* a, lapack_int lda, lapack_int k1,
                          lapack_int k2, const lapack_int* ipiv, lapack_int incx);
lapack_int LAPACKE_dlaswp_work(int matrix_layout, lapack_int n, double* a, lapack_int lda, lapack_int k1,
                               lapack_int k2, const lapack_int* ipiv, lapack_int incx);
lapack_int LAPACKE_slaswp(int matrix_layout, lapack_int n, float* a, lapack_int lda, lapack_int k1,
                          lapack_int k2, const lapack_int* ipiv, lapack_int incx);
lapack_int LAPACKE_slaswp_work(int matrix_layout, lapack_int n, float* a, lapack_int lda, lapack_int k1,
                               lapack_int k2, const lapack_int* ipiv, lapack_int incx);
/* LAPACKE/include/lapacke.h (dlag2s, slag2d) */
lapack_int LAPACKE_dlag2s(int matrix_layout, lapack_int m, lapack_int n, const double* a, lapack_int lda,
                          float* sa, lapack_int ldsa);
lapack_int LAPACKE_dlag2s_work(int matrix_layout, lapack_int m, lapack_int n, const double* a, lapack_int lda,
                               float* sa, lapack_int ldsa);
lapack_int LAPACKE_slag2d(int matrix_layout, lapack_int m, lapack_int n, const float* sa, lapack_int ldsa,
                          double* a, lapack_int lda);
/* LAPACKE/include/lapacke.h:469, 844, 1051 (dgecon, dgerfs, dgesvx) and their _work forms */
lapack_int LAPACKE_dgecon(int matrix_layout, char norm, lapack_int n, const double* a, lapack_int lda, double anorm,
                          double* rcond);
lapack_int LAPACKE_dgecon_work(int matrix_layout, char norm, lapack_int n, const double* a, lapack_int lda,
                               double anorm, double* rcond, double* work, lapack_int* iwork);
lapack_int LAPACKE_dgerfs(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const double* a,
                          lapack_int lda, const double* af, lapack_int ldaf, const lapack_int* ipiv, const double* b,
                          lapack_int ldb, double* x, lapack_int ldx, double* ferr, double* berr);
lapack_int LAPACKE_dgerfs_work(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const double* a,
                               lapack_int lda, const double* af, lapack_int ldaf, const lapack_int* ipiv,
                               const double* b, lapack_int ldb, double* x, lapack_int ldx, double* ferr,
                               double* berr, double* work, lapack_int* iwork);
lapack_int LAPACKE_dgesvx(int matrix_layout, char fact, char trans, lapack_int n, lapack_int nrhs, double* a,
                          lapack_int lda, double* af, lapack_int ldaf, lapack_int* ipiv, char* equed, double* r,
                          double* c, double* b, lapack_int ldb, double* x, lapack_int ldx, double* rcond,
                          double* ferr, double* berr, double* rpivot);
/* LAPACKE/include/lapacke.h:3030-3145, 8600 (dposv, dsposv, s/dpotrf, s/dpotrs) and their _work forms */
lapack_int LAPACKE_dpotrf(int matrix_layout, char uplo, lapack_int n, double* a, lapack_int lda);
lapack_int LAPACKE_dpotrf_work(int matrix_layout, char uplo, lapack_int n, double* a, lapack_int lda);
lapack_int LAPACKE_spotrf(int matrix_layout, char uplo, lapack_int n, float* a, lapack_int lda);
lapack_int LAPACKE_spotrf_work(int matrix_layout, char uplo, lapack_int n, float* a, lapack_int lda);
lapack_int LAPACKE_dpotrs(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, const double* a,
                          lapack_int lda, double* b, lapack_int ldb);
lapack_int LAPACKE_dpotrs_work(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, const double* a,
                               lapack_int lda, double* b, lapack_int ldb);
lapack_int LAPACKE_spotrs(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, const float* a, lapack_int lda,
                          float* b, lapack_int ldb);
lapack_int LAPACKE_spotrs_work(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, const float* a,
                               lapack_int lda, float* b, lapack_int ldb);
lapack_int LAPACKE_dposv(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                         double* b, lapack_int ldb);
lapack_int LAPACKE_dposv_work(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                              double* b, lapack_int ldb);
lapack_int LAPACKE_dsposv(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                          const double* b, lapack_int ldb, double* x, lapack_int ldx, lapack_int* iter);
lapack_int LAPACKE_dsposv_work(int matrix_layout, char uplo, lapack_int n, lapack_int nrhs, double* a, lapack_int lda,
                               const double* b, lapack_int ldb, double* x, lapack_int ldx, double* work,
                               float* swork, lapack_int* iter);
/* LAPACKE/include/lapacke.h (zgetrf, cgetrf, zgetrs, cgetrs, zgesv, cgesv,
 * zcgesv) and their _work forms; complex arrays as void*, so any
 * lapack_complex_double* / lapack_complex_float* passes. */
lapack_int LAPACKE_zgetrf(int matrix_layout, lapack_int m, lapack_int n, void* a, lapack_int lda, lapack_int* ipiv);
lapack_int LAPACKE_zgetrf_work(int matrix_layout, lapack_int m, lapack_int n, void* a, lapack_int lda,
                               lapack_int* ipiv);
lapack_int LAPACKE_cgetrf(int matrix_layout, lapack_int m, lapack_int n, void* a, lapack_int lda, lapack_int* ipiv);
lapack_int LAPACKE_cgetrf_work(int matrix_layout, lapack_int m, lapack_int n, void* a, lapack_int lda,
                               lapack_int* ipiv);
lapack_int LAPACKE_zgetrs(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const void* a, lapack_int lda,
                          const lapack_int* ipiv, void* b, lapack_int ldb);
lapack_int LAPACKE_zgetrs_work(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const void* a,
                               lapack_int lda, const lapack_int* ipiv, void* b, lapack_int ldb);
lapack_int LAPACKE_cgetrs(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const void* a, lapack_int lda,
                          const lapack_int* ipiv, void* b, lapack_int ldb);
lapack_int LAPACKE_cgetrs_work(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const void* a,
                               lapack_int lda, const lapack_int* ipiv, void* b, lapack_int ldb);
lapack_int LAPACKE_zgesv(int matrix_layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda, lapack_int* ipiv,
                         void* b, lapack_int ldb);
lapack_int LAPACKE_zgesv_work(int matrix_layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda,
                              lapack_int* ipiv, void* b, lapack_int ldb);
lapack_int LAPACKE_cgesv(int matrix_layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda, lapack_int* ipiv,
                         void* b, lapack_int ldb);
lapack_int LAPACKE_cgesv_work(int matrix_layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda,
                              lapack_int* ipiv, void* b, lapack_int ldb);
lapack_int LAPACKE_zcgesv(int matrix_layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda, lapack_int* ipiv,
                          const void* b, lapack_int ldb, void* x, lapack_int ldx, lapack_int* iter);
lapack_int LAPACKE_zcgesv_work(int matrix_layout, lapack_int n, lapack_int nrhs, void* a, lapack_int lda,
                               lapack_int* ipiv, const void* b, lapack_int ldb, void* x, lapack_int ldx, void* work,
                               void* swork, double* rwork, lapack_int* iter);
/* LAPACKE/include/lapacke.h:1153 (dgetri) and its _work form */
lapack_int LAPACKE_dgetri(int matrix_layout, lapack_int n, double* a, lapack_int lda, const lapack_int* ipiv);
lapack_int LAPACKE_dgetri_work(int matrix_layout, lapack_int n, double* a, lapack_int lda, const lapack_int* ipiv,
                               double* work, lapack_int lwork);
lapack_int LAPACKE_dgesvx_work(int matrix_layout, char fact, char trans, lapack_int n, lapack_int nrhs, double* a,
                               lapack_int lda, double* af, lapack_int ldaf, lapack_int* ipiv, char* equed, double* r,
                               double* c, double* b, lapack_int ldb, double* x, lapack_int ldx, double* rcond,
                               double* ferr, double* berr, double* work, lapack_int* iwork);
lapack_int LAPACKE_slag2d_work(int matrix_layout, lapack_int m, lapack_int n, const float* sa, lapack_int ldsa,
                               double* a, lapack_int lda);
/* LAPACKE/src/lapacke_nancheck.c:97-115 */
int LAPACKE_get_nancheck(void);
void LAPACKE_set_nancheck(int flag);
/* LAPACKE/utils/lapacke_xerbla.c */
void LAPACKE_xerbla(const char* name, lapack_int info);
/* LAPACKE/src/lapacke_alloc.c:57-61 */
void LAPACKE_set_alloc(void* (*malloc_fn)(size_t), void (*free_fn)(void*));
void* LAPACKE_malloc_proxy(size_t size);
void LAPACKE_free_proxy(void* ptr);

/* ---------------------------------------------------------------------
 * 3. Device-pointer entry points (no reference counterpart)
 *
 * Arrays are in GPU global memory of the current device, column-major.
 * The call queues its work on `stream` (NULL: the legacy default stream)
 * and returns when the result is complete; *info (host) receives the
 * LAPACK INFO.  Return value: 0 on success, a negative argument index for
 * an illegal argument (no xerbla_ call), or a positive CUDA / library
 * status code on a device failure.
 * ------------------------------------------------------------------- */
int gb300_dgetrf_dev(int m, int n, double* dA, int lda, int* dIpiv, int* info, void* stream);
int gb300_sgetrf_dev(int m, int n, float* dA, int lda, int* dIpiv, int* info, void* stream);
int gb300_dgetrs_dev(char trans, int n, int nrhs, const double* dA, int lda, const int* dIpiv, double* dB,
                     int ldb, void* stream);
int gb300_sgetrs_dev(char trans, int n, int nrhs, const float* dA, int lda, const int* dIpiv, float* dB,
                     int ldb, void* stream);
int gb300_dgesv_dev(int n, int nrhs, double* dA, int lda, int* dIpiv, double* dB, int ldb, int* info,
                    void* stream);
int gb300_dsgesv_dev(int n, int nrhs, double* dA, int lda, int* dIpiv, const double* dB, int ldb, double* dX,
                     int ldx, int* iter, int* info, void* stream);
/* DGECON on device memory (SRC/dgecon.f:124): dA holds the LU factors;
 * *rcond and *info are host outputs.  Returns 0, the negative index of an
 * illegal argument, or a positive device status. */
int gb300_dgecon_dev(char norm, int n, const double* dA, int lda, double anorm, double* rcond, int* info,
                     void* stream);
/* DLATRS on device memory (SRC/dlatrs.f:238): dA (n x n), dX and dCnorm
 * (n) are device arrays; *scale is a host output. */
int gb300_dlatrs_dev(char uplo, char trans, char diag, char normin, int n, const double* dA, int lda, double* dX,
                     double* scale, double* dCnorm, void* stream);
/* DGESVX on device memory (SRC/dgesvx.f:344): dA, dAF (n x n), dB, dX
 * (n x nrhs), dIpiv, dR, dC (n), dFerr, dBerr (nrhs) are device arrays;
 * *equed (in for FACT = 'F', out otherwise), *rcond, *rpvgrw (the
 * reference's WORK(1)) and *info are host values. */
int gb300_dgesvx_dev(char fact, char trans, int n, int nrhs, double* dA, int lda, double* dAF, int ldaf, int* dIpiv,
                     char* equed, double* dR, double* dC, double* dB, int ldb, double* dX, int ldx, double* rcond,
                     double* dFerr, double* dBerr, double* rpvgrw, int* info, void* stream);
/* DGETRI on device memory (SRC/dgetri.f:111): dA holds the LU factors
 * and receives inv(A); dIpiv on the device; *info host.  No workspace
 * argument: the library's scratch is stream ordered. */
int gb300_dgetri_dev(int n, double* dA, int lda, const int* dIpiv, int* info, void* stream);
/* Cholesky on device memory: DPOTRF (one triangle of dA, in place; *info
 * host), DPOTRS with those factors, DSPOSV (*iter, *info host). */
int gb300_dpotrf_dev(char uplo, int n, double* dA, int lda, int* info, void* stream);
int gb300_dpotrs_dev(char uplo, int n, int nrhs, const double* dA, int lda, double* dB, int ldb, void* stream);
int gb300_dsposv_dev(char uplo, int n, int nrhs, double* dA, int lda, const double* dB, int ldb, double* dX, int ldx,
                     int* iter, int* info, void* stream);
/* ZGETRF / ZGETRS / ZGESV on device memory (SRC/zgetrf.f:105,
 * SRC/zgetrs.f:118, SRC/zgesv.f:121): dA, dB hold (re, im) double pairs,
 * dIpiv is a device int array; INFO goes to the host int *info; the return
 * value is 0, the negative index of an illegal argument, or a CUDA status. */
int gb300_zgetrf_dev(int m, int n, void* dA, int lda, int* dIpiv, int* info, void* stream);
int gb300_zgetrs_dev(char trans, int n, int nrhs, const void* dA, int lda, const int* dIpiv, void* dB, int ldb,
                     void* stream);
int gb300_zgesv_dev(int n, int nrhs, void* dA, int lda, int* dIpiv, void* dB, int ldb, int* info, void* stream);
/* ZCGESV on device memory (SRC/zcgesv.f:197): ITER and INFO go to host ints. */
int gb300_zcgesv_dev(int n, int nrhs, void* dA, int lda, int* dIpiv, const void* dB, int ldb, void* dX, int ldx,
                     int* iter, int* info, void* stream);
/* DGERFS on device memory (SRC/dgerfs.f:181): dA, dAF (n x n), dB, dX
 * (n x nrhs), dIpiv (n) and dFerr, dBerr (nrhs) are device arrays; the
 * return value is 0, the negative index of an illegal argument as DGERFS
 * numbers them, or a positive device status. */
int gb300_dgerfs_dev(char trans, int n, int nrhs, const double* dA, int lda, const double* dAF, int ldaf,
                     const int* dIpiv, const double* dB, int ldb, double* dX, int ldx, double* dFerr,
                     double* dBerr, void* stream);
/* DGETRS on device memory that allocates nothing.  No counterpart in the
 * reference: it exists for callers that may not allocate GPU memory at the
 * point of the solve (a fixed device-memory budget reserved at start-up, a
 * latency-critical loop where an allocation could synchronise, code inside
 * an allocator callback).  Its scratch is one fixed array of about 1.1 MB
 * compiled into the library, held on every GPU that loads it until exit, so
 * it accepts n <= 16384 and n*nrhs <= 131072 and returns -100 for larger
 * problems.  The first call on a device looks up that array's address and
 * should come before any stream capture.  All calls share the array: calls
 * that overlap on the GPU race, so issue them one after another.  Each call
 * waits for its stream before it returns.  Same arguments and return codes
 * as gb300_dgetrs_dev otherwise; the solution agrees with that routine's to
 * rounding (this variant always runs the default FMA-form solve and does not
 * follow the exact-mode option). */
int gb300_dgetrs_noalloc(char trans, int n, int nrhs, const double* dA, int lda, const int* dIpiv, double* dB,
                         int ldb, void* stream);

/* Trailing-matrix update C := C - A*B, column-major (the DGEMM('N','N',
 * alpha=-1, beta=1) call of SRC/dgetrf.f:212-216 and its SGEMM twin).  The
 * FP32 form takes mode 0 (split-BF16x3 on the tensor cores) or 1 (FP32 FMA). */
int gb300_dgemm_update_dev(int m, int n, int k, const double* dA, int lda, const double* dB, int ldb, double* dC,
                           int ldc, void* stream);
int gb300_sgemm_update_dev(int mode, int m, int n, int k, const float* dA, int lda, const float* dB, int ldb,
                           float* dC, int ldc, void* stream);

/* Batched solves of many independent systems of uneven size (n <= 512,
 * nrhs <= 4) in one persistent launch; no reference counterpart (each
 * system is DGESV, SRC/dgesv.f, or DGETRF for the getrf form).  Arrays of
 * per-system device pointers and sizes, all in device memory; IPIV and
 * INFO per system (INFO = -1 for n > 512).  Asynchronous: nothing is
 * copied back and the host is not synchronised, so the call can be
 * captured into a CUDA graph. */
int gb300_dgesv_vbatched_dev(int batch, const int* d_n, const int* d_nrhs, double* const* dA_array, const int* d_lda,
                             int* const* dIpiv_array, double* const* dB_array, const int* d_ldb, int* d_info,
                             void* stream);
int gb300_sgesv_vbatched_dev(int batch, const int* d_n, const int* d_nrhs, float* const* dA_array, const int* d_lda,
                             int* const* dIpiv_array, float* const* dB_array, const int* d_ldb, int* d_info,
                             void* stream);
int gb300_dgetrf_vbatched_dev(int batch, const int* d_n, double* const* dA_array, const int* d_lda,
                              int* const* dIpiv_array, int* d_info, void* stream);
/* Panel width used for each 64-row size bucket (8 entries; dtype 0 double,
 * 1 float), as chosen by the autotuner (lapack_gb300.autotune_batched). */
int gb300_vbatched_set_nb(int dtype, const int* table);
int gb300_vbatched_get_nb(int dtype, int* table);
/* Instrumentation of the batched kernel, no reference counterpart: with
 * gb300_vbatched_profile(1) every later batched launch sums, per phase of
 * the per-system work, the SM cycles its CTAs spend (clock64 differences
 * of thread 0): [0] queue, [1] panel staging, [2] panel factorization,
 * [3] write-back and interchanges, [4] triangular solve of the U block row,
 * [5] trailing update, [6] the solve of the right-hand sides.
 * gb300_vbatched_profile_read copies the seven sums and clears them.
 * Returns the previous switch / 0, or -1 on a device error. */
int gb300_vbatched_profile(int on);
int gb300_vbatched_profile_read(unsigned long long* cycles);
/* Instrumentation of the FP32 cluster panel leaf (pushed exchange), no
 * reference counterpart: with gb300_leaf_profile(1) every later leaf adds
 * the SM cycles that CTA 0 spends in each step of its columns: [0] the
 * CTA's candidate reduction, [1] building and pushing its message, [2] the
 * wait for the cluster's messages, [3] the interchange, [4] the barrier
 * after it, [5] the update.  gb300_leaf_profile_read copies the six sums
 * and clears them.  Returns the previous switch / 0, or -1. */
int gb300_leaf_profile(int on);
/* Timeline of the look-ahead FP32 factorization and of the host-pointer
 * DSGESV's copies (test and bench hook, no reference counterpart): with
 * gb300_feed_trace(1) later calls record, on the device, the start of the
 * copies (kind 3), each chunk landed and converted (kind 2, idx = chunk),
 * each chunk taken into the factorization (kind 1, idx = chunk, aux = the
 * block-column step it joined at), each panel's start and end (kinds 6, 7,
 * idx = step), the next block column ready for the next panel (kind 5) and
 * each step's end (kind 0, idx = step, aux = columns taken in);
 * gb300_feed_trace_read returns up to cap records with their times in ms
 * after the first (waits for the last), or -1. */
int gb300_feed_trace(int on);
int gb300_feed_trace_read(int* kind, int* idx, int* aux, double* ms, int cap);
int gb300_leaf_profile_read(unsigned long long* cycles);

/* Adjoint of X = A^{-1} B from the stored factors (no reference counterpart;
 * the building blocks are DGETRS('T'), SRC/dgetrs.f:199-217, and
 * DGEMM('N','T'), BLAS/SRC/dgemm.f:363-383): gB = A^{-T} gX and, when dGA
 * is not NULL, gA = -gB X^T.  nrhs <= 16.  Synchronous. */
int gb300_dgesv_adjoint_dev(int n, int nrhs, const double* dLU, int ldlu, const int* dIpiv, const double* dX, int ldx,
                            const double* dGX, int ldgx, double* dGB, int ldgb, double* dGA, int ldga, void* stream);
/* The same for a uniform-size batch packed with element strides. */
int gb300_dgesv_adjoint_batched_dev(int batch, int n, int nrhs, const double* dLU, long long stride_lu,
                                    const int* dIpiv, long long stride_ipiv, const double* dX, long long stride_x,
                                    const double* dGX, long long stride_gx, double* dGB, long long stride_gb,
                                    double* dGA, long long stride_ga, void* stream);

/* Options: "exact" (0/1: products rounded separately, bitwise the
 * reference's operation order), "nb64" / "nb32" (outer block sizes),
 * "mixed" (0: BF16x3 tensor cores, 1: FP32 CUDA cores for DSGESV's FP32
 * factorization), "sgetrf" (same choice for SGETRF itself),
 * "panel_ctas64" / "panel_ctas32" (CTAs of the grid-wide panel kernel, 0:
 * all SMs), "cluster_panel" (FP32 leaves on one thread-block cluster: 2,
 * the default, shared-memory kernel exchanging each column's candidates
 * through a cluster barrier and remote loads; 3 the same kernel with the
 * exchange pushed to every CTA by remote asynchronous stores, faster alone
 * but slower beside the concurrent trailing update; 1 register kernel; 0
 * off),
 * "lookahead" (1: the
 * FP32 factorization factors block column k+1 on a second, high-priority
 * stream while the trailing update of block column k runs; 0: one stream),
 * "trsv_inv" (1: DSGESV's FP32 correction solves apply each 64 x 64
 * diagonal block as its inverse, formed in the solve; 0: substitution),
 * "gemm_ws" (1: the BF16x3 trailing update runs as a warp-specialised
 * multi-tile kernel; 0: one 128 x 128 tile per CTA), "gemm_tiles" (tiles
 * each CTA of the warp-specialised update takes, 4 by default; 0: one CTA
 * per SM),
 * "panel_fuse" (1: a node of the panel recursion whose halves are at most
 * 64 columns, U12 = L11^-1 A12 and A22 -= A21 U12, runs as one launch; 0:
 * two; bitwise the same), "feed" (1: the host-pointer dsgesv_ copies A in
 * column chunks on a second stream while the FP32 factorization takes each
 * chunk in as it lands; 0: the whole copy first; bitwise the same),
 * "feed_lazy" (test settings: 1, a landed chunk is taken in only when the
 * factorization needs it, which brings it up to date block column by block
 * column at once; 2, the next chunk is taken in at every step whether
 * landed or not, which exercises the catch-up spread over steps), "feed_catchup" (block columns of catch-up a landed chunk
 * taken in early gets per step, 8 by default; 0: all at once), "pool_keep" (1: the device's stream-ordered memory pool,
 * which this library's scratch comes from, keeps the memory it has grown to
 * for the rest of the process instead of returning it at every
 * synchronisation; read when the library first allocates on a device),
 * "ir_nan_guard" (0, the default, keeps DSGESV's stopping test exactly:
 * a residual of NaNs passes it, because RNRM.GT.XNRM*CTE is false for a
 * NaN (SRC/dsgesv.f:384-389), so a refinement that overflowed returns its
 * iterate with ITER > 0; 1 treats a NaN or infinity in the iterate or the
 * residual as DLAG2S treats an overflow: ITER = -2 and the FP64
 * factorization).
 * Returns the previous value, or -1 for an unknown name.  Not thread-safe:
 * set at start-up. */
int gb300_set_option(const char* name, int value);
int gb300_get_option(const char* name);
/* Reads (and with clear=1 resets) the device status word that kernels with
 * bounded waits set when a wait runs out: 0 means none did. */
int gb300_status(int clear);
/* xerbla_ capture: with on=1, illegal-argument reports are recorded instead
 * of stopping the program; gb300_xerbla_last returns the last INFO and
 * copies the routine name. */
void gb300_xerbla_capture(int on);
int gb300_xerbla_last(char* name, int cap);
const char* gb300_version(void);

/* Instrumentation (no reference counterpart).  gb300_launch_count: kernels
 * this library has launched so far in the process.  With profiling enabled,
 * every launch of the timed kernel classes is bracketed by CUDA events on
 * its own stream; gb300_prof_read sums, for one class (0 FP64 update, 1
 * FP32 update, 2 BF16x3 update, 3 panel, 4 row interchanges, 5 TRSM, 6
 * triangular solves, 7 FP64 residual, 8 other), the event time in ms, the
 * algorithmic flops and bytes, and the launch count.  gb300_prof_mask
 * limits the bracketed classes to the bits set in mask (bit k = class k;
 * default all), so that a timed run can carry events around one class only;
 * returns the previous mask. */
long long gb300_launch_count(void);
int gb300_prof_enable(int on);
unsigned gb300_prof_mask(unsigned mask);
void gb300_prof_reset(void);
int gb300_prof_read(int kind, double* ms, double* flops, double* bytes, long long* launches);
/* Measured arithmetic throughput of the current GPU in TFLOP/s: 0 FP64 FMA,
 * 1 FP32 FMA, 2 FP64 tensor core (mma.sync m8n8k4), 3 FP64 tensor core
 * (mma.sync m16n8k16); -1 for another value.  No reference counterpart. */
double gb300_probe_peak(int which);
/* Microseconds per iteration of the skeleton of one cluster-panel column
 * (two CTA barriers around a cluster-wide exchange of 16-byte messages) on
 * one cluster of `ctas` CTAs: mode 0 the pushed exchange (st.async counted
 * on the receivers' mbarriers), 1 a cluster barrier.  Negative on an error.
 * No reference counterpart: a measurement of the latency floor of the
 * FP32 panel leaf. */
double gb300_probe_cluster_exchange(int ctas, int mode, int iters);

#ifdef __cplusplus
}
#endif
#endif /* LAPACK_GB300_H */
