/* Test infrastructure only (oracle/_ref build): forwards the Fortran LAPACK entry points
 * that the reference smartpca calls (src/eigensrc/eigx.c:107 dspev_, src/nicksrc/linsubs.c
 * dpotrf_/dgetrf_/dgetri_/dgetrs_/dsygv_) to the scipy-bundled OpenBLAS, which exports
 * them under a `scipy_` prefix with 32-bit integers. */
typedef int lapack_int;

void scipy_dspev_(char *, char *, lapack_int *, double *, double *, double *,
                  lapack_int *, double *, lapack_int *);
void scipy_dpotrf_(char *, lapack_int *, double *, lapack_int *, lapack_int *);
void scipy_dgetrf_(lapack_int *, lapack_int *, double *, lapack_int *, lapack_int *,
                   lapack_int *);
void scipy_dgetri_(lapack_int *, double *, lapack_int *, lapack_int *, double *,
                   lapack_int *, lapack_int *);
void scipy_dgetrs_(char *, lapack_int *, lapack_int *, double *, lapack_int *,
                   lapack_int *, double *, lapack_int *, lapack_int *);
void scipy_dsygv_(lapack_int *, char *, char *, lapack_int *, double *, lapack_int *,
                  double *, lapack_int *, double *, double *, lapack_int *, lapack_int *);

void dspev_(char *jobz, char *uplo, lapack_int *n, double *ap, double *w, double *z,
            lapack_int *ldz, double *work, lapack_int *info)
{
  scipy_dspev_(jobz, uplo, n, ap, w, z, ldz, work, info);
}

void dpotrf_(char *uplo, lapack_int *n, double *a, lapack_int *lda, lapack_int *info)
{
  scipy_dpotrf_(uplo, n, a, lda, info);
}

void dgetrf_(lapack_int *m, lapack_int *n, double *a, lapack_int *lda, lapack_int *ipiv,
             lapack_int *info)
{
  scipy_dgetrf_(m, n, a, lda, ipiv, info);
}

void dgetri_(lapack_int *n, double *a, lapack_int *lda, lapack_int *ipiv, double *work,
             lapack_int *lwork, lapack_int *info)
{
  scipy_dgetri_(n, a, lda, ipiv, work, lwork, info);
}

void dgetrs_(char *trans, lapack_int *n, lapack_int *nrhs, double *a, lapack_int *lda,
             lapack_int *ipiv, double *b, lapack_int *ldb, lapack_int *info)
{
  scipy_dgetrs_(trans, n, nrhs, a, lda, ipiv, b, ldb, info);
}

void dsygv_(lapack_int *itype, char *jobz, char *uplo, lapack_int *n, double *a,
            lapack_int *lda, double *b, lapack_int *ldb, double *w, double *work,
            lapack_int *lwork, lapack_int *info)
{
  scipy_dsygv_(itype, jobz, uplo, n, a, lda, b, ldb, w, work, lwork, info);
}
