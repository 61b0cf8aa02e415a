/* TEST INFRASTRUCTURE ONLY.  Prepended (g++ -include) to the hsolve lines
 * extracted from fastSolver2's src/tasks/leaf_solve.cc so that they compile
 * without Legion: it supplies the headers those lines use and the
 * blas::dgemm_ / lapack::dgesv_ declarations of include/lapack_blas.hpp:28-57.
 * The two symbols resolve to forwarding stubs in ref_blas.cc. */
#include <cassert>
#include <cmath>
#include <cstdlib>
#include <iostream>
namespace blas {
extern "C" void dgemm_(char *transa, char *transb, int *m, int *n, int *k,
                       double *alpha, double *A, int *lda, double *B, int *ldb,
                       double *beta, double *C, int *ldc);
}
namespace lapack {
extern "C" void dgesv_(int *N, int *NRHS, double *A, int *LDA, int *IPIV,
                       double *B, int *LDB, int *INFO);
}
