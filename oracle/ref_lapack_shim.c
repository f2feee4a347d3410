/*
 * LAPACK forwarding shim for building the reference Griffon (test infrastructure only).
 *
 * The reference links the system LAPACK (setup.py:112); this image has none, but scipy ships OpenBLAS with
 * the Fortran LAPACK entry points exported under a "scipy_" prefix. These three wrappers give the reference
 * its dgetrf_/dgetrs_/dgeev_ (blas_lapack_kernels.h:95-180) by calling the scipy-exported ones.
 */
extern void scipy_dgetrf_(const int *, const int *, double *, const int *, int *, int *);
extern void scipy_dgetrs_(const char *, const int *, const int *, const double *, const int *, const int *,
                          double *, const int *, int *, long);
extern void scipy_dgeev_(const char *, const char *, const int *, double *, const int *, double *, double *,
                         double *, const int *, double *, const int *, double *, int *, int *, long, long);

void dgetrf_(const int *m, const int *n, double *a, const int *lda, int *ipiv, int *info)
{
  scipy_dgetrf_(m, n, a, lda, ipiv, info);
}

void dgetrs_(const char *t, const int *n, const int *nrhs, const double *a, const int *lda, const int *ipiv,
             double *b, const int *ldb, int *info)
{
  scipy_dgetrs_(t, n, nrhs, a, lda, ipiv, b, ldb, info, 1);
}

void dgeev_(const char *jl, const char *jr, const int *n, double *a, const int *lda, double *wr, double *wi,
            double *vl, const int *ldvl, double *vr, const int *ldvr, double *work, int *lwork, int *info)
{
  scipy_dgeev_(jl, jr, n, a, lda, wr, wi, vl, ldvl, vr, ldvr, work, lwork, info, 1, 1);
}
