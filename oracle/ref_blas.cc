/* TEST INFRASTRUCTURE ONLY.  BLAS/LAPACK provider for the verbatim
 * reference hsolve build: dgemm_/dgesv_ forward to the LP64 routines that
 * scipy's bundled OpenBLAS exports under the scipy_ prefix, and ref_hsolve
 * gives the C++-linkage hsolve (src/tasks/leaf_solve.cc:73-154) a C name. */
extern "C" {
void scipy_dgemm_(char *, char *, int *, int *, int *, double *, double *,
                  int *, double *, int *, double *, double *, int *);
void scipy_dgesv_(int *, int *, double *, int *, int *, double *, int *, int *);
void dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *alpha,
            double *A, int *lda, double *B, int *ldb, double *beta, double *C,
            int *ldc) {
  scipy_dgemm_(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
void dgesv_(int *N, int *NRHS, double *A, int *LDA, int *IPIV, double *B,
            int *LDB, int *INFO) {
  scipy_dgesv_(N, NRHS, A, LDA, IPIV, B, LDB, INFO);
}
}
void hsolve(int nrow, int nrhs, int rank, int nPart, int LD, double *K,
            double *U, double *V);
extern "C" void ref_hsolve(int nrow, int nrhs, int rank, int nPart, int LD,
                           double *K, double *U, double *V) {
  hsolve(nrow, nrhs, rank, nPart, LD, K, U, V);
}
