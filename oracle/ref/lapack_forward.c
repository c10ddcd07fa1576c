/* Forward the five Fortran-ABI LAPACK/BLAS symbols the reference's
 * cpp/blas_wrapper.cpp declares (dgesvd_, dgemm_, dgemv_, dgetrf_, dgetrs_)
 * to the copies exported by scipy's bundled OpenBLAS, whose names carry a
 * "scipy_" prefix.  Test infrastructure for oracle/_ref only. */
void scipy_dgetrf_(int*, int*, double*, int*, int*, int*);
void scipy_dgetrs_(char*, int*, int*, double*, int*, int*, double*, int*, int*);
void scipy_dgesvd_(char*, char*, int*, int*, double*, int*, double*, double*, int*,
                   double*, int*, double*, int*, int*);
void scipy_dgemm_(char*, char*, int*, int*, int*, double*, double*, int*, double*,
                  int*, double*, double*, int*);
void scipy_dgemv_(char*, int*, int*, double*, double*, int*, double*, int*, double*,
                  double*, int*);

void dgetrf_(int* m, int* n, double* a, int* lda, int* ipiv, int* info)
{ scipy_dgetrf_(m, n, a, lda, ipiv, info); }
void dgetrs_(char* t, int* n, int* nrhs, double* a, int* lda, int* ipiv, double* b,
             int* ldb, int* info)
{ scipy_dgetrs_(t, n, nrhs, a, lda, ipiv, b, ldb, info); }
void dgesvd_(char* ju, char* jvt, int* m, int* n, double* a, int* lda, double* s,
             double* u, int* ldu, double* vt, int* ldvt, double* work, int* lwork,
             int* info)
{ scipy_dgesvd_(ju, jvt, m, n, a, lda, s, u, ldu, vt, ldvt, work, lwork, info); }
void dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* al, double* a, int* lda,
            double* b, int* ldb, double* be, double* c, int* ldc)
{ scipy_dgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc); }
void dgemv_(char* t, int* m, int* n, double* al, double* a, int* lda, double* x,
            int* incx, double* be, double* y, int* incy)
{ scipy_dgemv_(t, m, n, al, a, lda, x, incx, be, y, incy); }
