/*
 * hodlr_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, single-precision-free (FP64) restatement of fastSolver2's HODLR
 * leaf-solve / capacitance / low-rank-update path and of the netlib LAPACK/BLAS
 * routines it calls.  It is the checker for the CUDA path: only tests/, the
 * smoke() entry point and bench.py's cpu_baseline / --impl reference leg load
 * it.  The product library (fastsolver2_gb300/csrc) never calls it.
 *
 * Everything is column-major with explicit leading dimensions, as in the
 * reference (src/ptr_matrix.cc:29-37).  Pivot vectors use the LAPACK
 * convention: ipiv[i] is the 1-based row that row i+1 was swapped with.
 *
 * Compile with -ffp-contract=off so x86_64 and aarch64 builds give the same
 * bits (GCC contracts a*b+c into FMA by default on aarch64).
 *
 * Sources restated (file:line inside the fastSolver2 tree):
 *   drand48 generators ........ src/ptr_matrix.cc:62-71, src/matrix.cc:51-102,250-297
 *   dense leaf block .......... src/tasks/dense_block.cc:63-75, src/ptr_matrix.cc:141-164
 *   hsolve .................... src/tasks/leaf_solve.cc:73-154
 *   capacitance solve ......... src/tasks/node_solve.cc:60-81
 *   DGESV/DGETRF/DGETRF2 ...... netlib_blas/dgesv.f, dgetrf.f:109, dgetrf2.f:114
 *   DGETRS/DLASWP/DTRSM ....... netlib_blas/dgetrs.f:122, dlaswp.f:115, dtrsm.f:182
 *   DGEMM/IDAMAX/DSCAL ........ netlib_blas/dgemm.f:188, idamax.f:52, dscal.f
 *   ILAENV block size (64) .... netlib_blas/ilaenv.f:272-278
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_API __attribute__((visibility("default")))
#define A_(i, j) A[(int64_t)(i) + (int64_t)(j) * lda]
#define B_(i, j) B[(int64_t)(i) + (int64_t)(j) * ldb]
#define C_(i, j) C[(int64_t)(i) + (int64_t)(j) * ldc]

/* ------------------------------------------------------------------------ */
/* drand48 generators (src/ptr_matrix.cc:62-71, src/matrix.cc:250-297)      */
/* ------------------------------------------------------------------------ */

/* Per-partition seeds, as Matrix::rand() draws them (src/matrix.cc:271-280)
 * with the time(NULL)-based master seed replaced by a fixed one. */
ORC_API void orc_seeds(long master, int n, long *out) {
  struct drand48_data buf;
  srand48_r(master, &buf);
  for (int i = 0; i < n; ++i) {
    long s;
    lrand48_r(&buf, &s);
    out[i] = s;
  }
}

/* PtrMatrix::rand(seed, offset) (src/ptr_matrix.cc:62-71): a rows x cols
 * column-major block filled in row-major order (for i rows, for j cols). */
ORC_API void orc_rand_block(long seed, int rows, int cols, int64_t lda,
                            double *A, int offset) {
  struct drand48_data buf;
  srand48_r(seed, &buf);
  for (int i = 0; i < rows; ++i)
    for (int j = 0; j < cols; ++j) {
      drand48_r(&buf, &A_(i, j));
      A_(i, j) += offset;
    }
}

/* Matrix(base, level, col).rand() (src/matrix.cc:271-297): 2^level row
 * blocks of `base` rows, block k filled from seeds[k]. */
ORC_API void orc_rand_matrix(const long *seeds, int nPart, int base, int cols,
                             double *A, int offset) {
  int64_t lda = (int64_t)nPart * base;
  for (int k = 0; k < nPart; ++k)
    orc_rand_block(seeds[k], base, cols, lda, A + (int64_t)k * base, offset);
}

/* DenseBlockTask (src/tasks/dense_block.cc:63-75) + PtrMatrix::gemm(U,V,D,K)
 * (src/ptr_matrix.cc:141-164): leaf k of the KTree region (rows k*m..,
 * columns 0..m, LD = ldk) is U_k V_k^T + diag(D_k).  U, V and D are
 * regenerated from the per-leaf seeds exactly as the task does. */
void orc_dgemm(char ta, char tb, int m, int n, int k, double alpha,
               const double *A, int64_t lda, const double *B, int64_t ldb,
               double beta, double *C, int64_t ldc);

ORC_API void orc_dense_blocks(const long *useeds, const long *vseeds,
                              const long *dseeds, int nleaf, int m, int rank,
                              int offset, double *K, int64_t ldk) {
  double *U = (double *)malloc(sizeof(double) * m * rank);
  double *V = (double *)malloc(sizeof(double) * m * rank);
  double *D = (double *)malloc(sizeof(double) * m);
  for (int k = 0; k < nleaf; ++k) {
    orc_rand_block(useeds[k], m, rank, m, U, 0);
    orc_rand_block(vseeds[k], m, rank, m, V, 0);
    orc_rand_block(dseeds[k], m, 1, m, D, offset);
    double *Kk = K + (int64_t)k * m;
    orc_dgemm('n', 't', m, m, rank, 1.0, U, m, V, m, 0.0, Kk, ldk);
    for (int i = 0; i < m; ++i) Kk[i + (int64_t)i * ldk] += D[i];
  }
  free(U);
  free(V);
  free(D);
}

/* ------------------------------------------------------------------------ */
/* netlib BLAS restatement                                                   */
/* ------------------------------------------------------------------------ */

/* IDAMAX (netlib_blas/idamax.f:52): first index of max |x|, 1-based. */
ORC_API int orc_idamax(int n, const double *x) {
  if (n < 1) return 0;
  int idx = 1;
  double dmax = fabs(x[0]);
  for (int i = 2; i <= n; ++i)
    if (fabs(x[i - 1]) > dmax) {
      idx = i;
      dmax = fabs(x[i - 1]);
    }
  return idx;
}

/* DSCAL with unit stride. */
static void orc_dscal(int n, double a, double *x) {
  for (int i = 0; i < n; ++i) x[i] = a * x[i];
}

/* DGEMM (netlib_blas/dgemm.f:188), same loop order per transpose case. */
ORC_API void orc_dgemm(char ta, char tb, int m, int n, int k, double alpha,
                       const double *A, int64_t lda, const double *B,
                       int64_t ldb, double beta, double *C, int64_t ldc) {
  int nota = (ta == 'n' || ta == 'N');
  int notb = (tb == 'n' || tb == 'N');
  if (m == 0 || n == 0 || ((alpha == 0.0 || k == 0) && beta == 1.0)) return;
  if (alpha == 0.0) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) C_(i, j) = (beta == 0.0) ? 0.0 : beta * C_(i, j);
    return;
  }
  if (notb) {
    if (nota) {
      for (int j = 0; j < n; ++j) {
        if (beta == 0.0) {
          for (int i = 0; i < m; ++i) C_(i, j) = 0.0;
        } else if (beta != 1.0) {
          for (int i = 0; i < m; ++i) C_(i, j) = beta * C_(i, j);
        }
        for (int l = 0; l < k; ++l) {
          double temp = alpha * B_(l, j);
          for (int i = 0; i < m; ++i) C_(i, j) = C_(i, j) + temp * A_(i, l);
        }
      }
    } else {
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) {
          double temp = 0.0;
          for (int l = 0; l < k; ++l) temp = temp + A_(l, i) * B_(l, j);
          C_(i, j) = (beta == 0.0) ? alpha * temp : alpha * temp + beta * C_(i, j);
        }
    }
  } else {
    if (nota) {
      for (int j = 0; j < n; ++j) {
        if (beta == 0.0) {
          for (int i = 0; i < m; ++i) C_(i, j) = 0.0;
        } else if (beta != 1.0) {
          for (int i = 0; i < m; ++i) C_(i, j) = beta * C_(i, j);
        }
        for (int l = 0; l < k; ++l) {
          double temp = alpha * B_(j, l);
          for (int i = 0; i < m; ++i) C_(i, j) = C_(i, j) + temp * A_(i, l);
        }
      }
    } else {
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) {
          double temp = 0.0;
          for (int l = 0; l < k; ++l) temp = temp + A_(l, i) * B_(j, l);
          C_(i, j) = (beta == 0.0) ? alpha * temp : alpha * temp + beta * C_(i, j);
        }
    }
  }
}

/* DTRSM, SIDE='L', alpha = 1 (netlib_blas/dtrsm.f:182): the four cases
 * DGETRS needs.  uplo 'L'/'U', trans 'N'/'T', unit diagonal iff uplo=='L'. */
static void orc_dtrsm_left(char uplo, char trans, int m, int n,
                           const double *A, int64_t lda, double *B,
                           int64_t ldb) {
  if (m == 0 || n == 0) return;
  int upper = (uplo == 'U');
  int nounit = upper; /* L is unit lower, U is non-unit upper */
  if (trans == 'N') {
    if (upper) {
      for (int j = 0; j < n; ++j)
        for (int k = m - 1; k >= 0; --k)
          if (B_(k, j) != 0.0) {
            if (nounit) B_(k, j) = B_(k, j) / A_(k, k);
            for (int i = 0; i < k; ++i) B_(i, j) = B_(i, j) - B_(k, j) * A_(i, k);
          }
    } else {
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < m; ++k)
          if (B_(k, j) != 0.0) {
            if (nounit) B_(k, j) = B_(k, j) / A_(k, k);
            for (int i = k + 1; i < m; ++i) B_(i, j) = B_(i, j) - B_(k, j) * A_(i, k);
          }
    }
  } else {
    if (upper) {
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) {
          double temp = B_(i, j);
          for (int k = 0; k < i; ++k) temp = temp - A_(k, i) * B_(k, j);
          if (nounit) temp = temp / A_(i, i);
          B_(i, j) = temp;
        }
    } else {
      for (int j = 0; j < n; ++j)
        for (int i = m - 1; i >= 0; --i) {
          double temp = B_(i, j);
          for (int k = i + 1; k < m; ++k) temp = temp - A_(k, i) * B_(k, j);
          if (nounit) temp = temp / A_(i, i);
          B_(i, j) = temp;
        }
    }
  }
}

/* DLASWP (netlib_blas/dlaswp.f:115) on columns [0,n); k1..k2 are 1-based. */
ORC_API void orc_dlaswp(int n, double *A, int64_t lda, int k1, int k2,
                        const int *ipiv, int incx) {
  if (incx == 0) return;
  for (int j = 0; j < n; ++j) {
    if (incx > 0) {
      for (int i = k1; i <= k2; ++i) {
        int ip = ipiv[i - 1];
        if (ip != i) {
          double t = A_(i - 1, j);
          A_(i - 1, j) = A_(ip - 1, j);
          A_(ip - 1, j) = t;
        }
      }
    } else {
      for (int i = k2; i >= k1; --i) {
        int ip = ipiv[i - 1];
        if (ip != i) {
          double t = A_(i - 1, j);
          A_(i - 1, j) = A_(ip - 1, j);
          A_(ip - 1, j) = t;
        }
      }
    }
  }
}

/* DGETRF2 (netlib_blas/dgetrf2.f:114): recursive panel LU.  Returns INFO. */
ORC_API int orc_dgetrf2(int m, int n, double *A, int64_t lda, int *ipiv) {
  int info = 0;
  if (m == 0 || n == 0) return 0;
  if (m == 1) {
    ipiv[0] = 1;
    if (A_(0, 0) == 0.0) info = 1;
  } else if (n == 1) {
    const double sfmin = 2.2250738585072014e-308; /* DLAMCH('S') */
    int i = orc_idamax(m, &A_(0, 0));
    ipiv[0] = i;
    if (A_(i - 1, 0) != 0.0) {
      if (i != 1) {
        double t = A_(0, 0);
        A_(0, 0) = A_(i - 1, 0);
        A_(i - 1, 0) = t;
      }
      if (fabs(A_(0, 0)) >= sfmin) {
        orc_dscal(m - 1, 1.0 / A_(0, 0), &A_(1, 0));
      } else {
        for (int q = 1; q < m; ++q) A_(q, 0) = A_(q, 0) / A_(0, 0);
      }
    } else {
      info = 1;
    }
  } else {
    int n1 = (m < n ? m : n) / 2;
    int n2 = n - n1;
    int iinfo = orc_dgetrf2(m, n1, A, lda, ipiv);
    if (info == 0 && iinfo > 0) info = iinfo;
    orc_dlaswp(n2, &A_(0, n1), lda, 1, n1, ipiv, 1);
    orc_dtrsm_left('L', 'N', n1, n2, A, lda, &A_(0, n1), lda);
    orc_dgemm('n', 'n', m - n1, n2, n1, -1.0, &A_(n1, 0), lda, &A_(0, n1), lda,
              1.0, &A_(n1, n1), lda);
    iinfo = orc_dgetrf2(m - n1, n2, &A_(n1, n1), lda, ipiv + n1);
    if (info == 0 && iinfo > 0) info = iinfo + n1;
    int mn = m < n ? m : n;
    for (int q = n1; q < mn; ++q) ipiv[q] += n1;
    orc_dlaswp(n1, A, lda, n1 + 1, mn, ipiv, 1);
  }
  return info;
}

/* DGETRF (netlib_blas/dgetrf.f:109) with the ILAENV block size NB = 64. */
ORC_API int orc_dgetrf(int m, int n, double *A, int64_t lda, int *ipiv) {
  const int nb = 64;
  int info = 0;
  if (m == 0 || n == 0) return 0;
  int mn = m < n ? m : n;
  if (nb <= 1 || nb >= mn) return orc_dgetrf2(m, n, A, lda, ipiv);
  for (int j = 1; j <= mn; j += nb) {
    int jb = (mn - j + 1) < nb ? (mn - j + 1) : nb;
    int iinfo = orc_dgetrf2(m - j + 1, jb, &A_(j - 1, j - 1), lda, ipiv + j - 1);
    if (info == 0 && iinfo > 0) info = iinfo + j - 1;
    int hi = (m < j + jb - 1) ? m : j + jb - 1;
    for (int i = j; i <= hi; ++i) ipiv[i - 1] = j - 1 + ipiv[i - 1];
    orc_dlaswp(j - 1, A, lda, j, j + jb - 1, ipiv, 1);
    if (j + jb <= n) {
      orc_dlaswp(n - j - jb + 1, &A_(0, j + jb - 1), lda, j, j + jb - 1, ipiv, 1);
      orc_dtrsm_left('L', 'N', jb, n - j - jb + 1, &A_(j - 1, j - 1), lda,
                     &A_(j - 1, j + jb - 1), lda);
      if (j + jb <= m)
        orc_dgemm('n', 'n', m - j - jb + 1, n - j - jb + 1, jb, -1.0,
                  &A_(j + jb - 1, j - 1), lda, &A_(j - 1, j + jb - 1), lda, 1.0,
                  &A_(j + jb - 1, j + jb - 1), lda);
    }
  }
  return info;
}

/* DGETRS (netlib_blas/dgetrs.f:122), trans = 'N' or 'T'. */
ORC_API void orc_dgetrs(char trans, int n, int nrhs, const double *A,
                        int64_t lda, const int *ipiv, double *B, int64_t ldb) {
  if (n == 0 || nrhs == 0) return;
  if (trans == 'N' || trans == 'n') {
    orc_dlaswp(nrhs, B, ldb, 1, n, ipiv, 1);
    orc_dtrsm_left('L', 'N', n, nrhs, A, lda, B, ldb);
    orc_dtrsm_left('U', 'N', n, nrhs, A, lda, B, ldb);
  } else {
    orc_dtrsm_left('U', 'T', n, nrhs, A, lda, B, ldb);
    orc_dtrsm_left('L', 'T', n, nrhs, A, lda, B, ldb);
    orc_dlaswp(nrhs, B, ldb, 1, n, ipiv, -1);
  }
}

/* DGESV (netlib_blas/dgesv.f). */
ORC_API int orc_dgesv(int n, int nrhs, double *A, int64_t lda, int *ipiv,
                      double *B, int64_t ldb) {
  int info = orc_dgetrf(n, n, A, lda, ipiv);
  if (info == 0) orc_dgetrs('N', n, nrhs, A, lda, ipiv, B, ldb);
  return info;
}

/* ------------------------------------------------------------------------ */
/* hsolve (src/tasks/leaf_solve.cc:73-154), reference structure: one V for   */
/* every level, U chunks living in the same region as the right-hand side.   */
/* Returns 0, or the LAPACK INFO of the first failing dgesv.                 */
/* ------------------------------------------------------------------------ */
ORC_API int orc_hsolve(int nrow, int nrhs, int rank, int nPart, int64_t LD,
                       double *K, double *U, double *V) {
  if (nPart == 1) {
    int *ipiv = (int *)malloc(sizeof(int) * (nrow > 0 ? nrow : 1));
    int info = orc_dgesv(nrow, nrhs, K, LD, ipiv, U, LD);
    free(ipiv);
    return info;
  }
  double *d0 = U, *d1 = U + nrow / 2;
  double *V0 = V, *V1 = V + nrow / 2;
  double *u0 = d0 + (int64_t)nrhs * LD, *u1 = d1 + (int64_t)nrhs * LD;
  int info = orc_hsolve(nrow / 2, nrhs + rank, rank, nPart / 2, LD, K, d0, V0);
  if (info) return info;
  info = orc_hsolve(nrow / 2, nrhs + rank, rank, nPart / 2, LD, K + nrow / 2, d1, V1);
  if (info) return info;
  int S_size = 2 * rank;
  double *S = (double *)calloc((size_t)S_size * S_size, sizeof(double));
  double *RHS = (double *)malloc(sizeof(double) * S_size * (nrhs > 0 ? nrhs : 1));
  int *ipiv = (int *)malloc(sizeof(int) * S_size);
  for (int i = 0; i < S_size; ++i) S[S_size * i + i] = 1.0;
  double *V0Tu0 = S + S_size / 2;
  double *V1Tu1 = S + S_size / 2 * S_size;
  double *V0Td0 = RHS + S_size / 2;
  double *V1Td1 = RHS;
  int h = nrow / 2;
  orc_dgemm('t', 'n', rank, rank, h, 1.0, V0, LD, u0, LD, 0.0, V0Tu0, S_size);
  orc_dgemm('t', 'n', rank, rank, h, 1.0, V1, LD, u1, LD, 0.0, V1Tu1, S_size);
  orc_dgemm('t', 'n', rank, nrhs, h, 1.0, V0, LD, d0, LD, 0.0, V0Td0, S_size);
  orc_dgemm('t', 'n', rank, nrhs, h, 1.0, V1, LD, d1, LD, 0.0, V1Td1, S_size);
  info = orc_dgesv(S_size, nrhs, S, S_size, ipiv, RHS, S_size);
  if (info == 0) {
    double *eta0 = V1Td1, *eta1 = V0Td0;
    orc_dgemm('n', 'n', h, nrhs, rank, -1.0, u0, LD, eta0, S_size, 1.0, d0, LD);
    orc_dgemm('n', 'n', h, nrhs, rank, -1.0, u1, LD, eta1, S_size, 1.0, d1, LD);
  } else {
    info = -1000 - info; /* singular capacitance system */
  }
  free(S);
  free(RHS);
  free(ipiv);
  return info;
}

/* ------------------------------------------------------------------------ */
/* Generalised HODLR (per-level U^(l), V^(l), optional diag(s^(l))), with    */
/* the factorisation kept.  The recursion, column layout and capacitance     */
/* system are those of hsolve; a node at depth l couples its children c0,c1  */
/* through A[c0,c1] = U^(l)_c0 diag(s^(l)) V^(l)_c1^T and                    */
/* A[c1,c0] = U^(l)_c1 diag(s^(l)) V^(l)_c0^T.                               */
/*                                                                           */
/* Work array W (N x (nrhs + L*r), ld ldw): on entry [B | U^(0) | ... ],      */
/* on exit [X | Utilde^(0) | ...] exactly as hsolve leaves the UTree region. */
/* Optional outputs (NULL to skip): leaf pivots [nleaf*m], capacitance LU    */
/* [nnode][2r][2r] col-major and pivots [nnode][2r]; node id of position p   */
/* at depth l is (2^l - 1) + p.                                              */
/* ------------------------------------------------------------------------ */
typedef struct {
  int leaf, levels, rank;
  double *K;
  int64_t ldk;
  const double *const *V; /* V[l]: N x r, ld ldv */
  int64_t ldv;
  const double *const *s; /* s[l]: r entries, or NULL */
  int *leaf_ipiv;
  double *cap_lu;
  int *cap_ipiv;
} orc_hodlr;

static int orc_hgen_rec(const orc_hodlr *h, int depth, int64_t row0, int nrow,
                        int nrhs, double *W, int64_t ldw, int pos) {
  const int r = h->rank;
  if (depth == h->levels) {
    int leaf_id = pos;
    int *ipiv = h->leaf_ipiv ? h->leaf_ipiv + (int64_t)leaf_id * h->leaf
                             : (int *)malloc(sizeof(int) * nrow);
    double *Kk = h->K + row0;
    int info = orc_dgetrf(nrow, nrow, Kk, h->ldk, ipiv);
    if (info == 0) orc_dgetrs('N', nrow, nrhs, Kk, h->ldk, ipiv, W + row0, ldw);
    if (!h->leaf_ipiv) free(ipiv);
    return info ? 1 + leaf_id : 0;
  }
  int half = nrow / 2;
  int info = orc_hgen_rec(h, depth + 1, row0, half, nrhs + r, W, ldw, 2 * pos);
  if (info) return info;
  info = orc_hgen_rec(h, depth + 1, row0 + half, half, nrhs + r, W, ldw, 2 * pos + 1);
  if (info) return info;
  const double *V = h->V[depth];
  const double *s = h->s ? h->s[depth] : NULL;
  const double *V0 = V + row0, *V1 = V + row0 + half;
  double *d0 = W + row0, *d1 = W + row0 + half;
  double *u0 = d0 + (int64_t)nrhs * ldw, *u1 = d1 + (int64_t)nrhs * ldw;
  int S_size = 2 * r;
  double *S = (double *)calloc((size_t)S_size * S_size, sizeof(double));
  double *RHS = (double *)malloc(sizeof(double) * S_size * (nrhs > 0 ? nrhs : 1));
  int *ipiv = (int *)malloc(sizeof(int) * S_size);
  for (int i = 0; i < S_size; ++i) S[S_size * i + i] = 1.0;
  orc_dgemm('t', 'n', r, r, half, 1.0, V0, h->ldv, u0, ldw, 0.0, S + r, S_size);
  orc_dgemm('t', 'n', r, r, half, 1.0, V1, h->ldv, u1, ldw, 0.0, S + (int64_t)r * S_size, S_size);
  orc_dgemm('t', 'n', r, nrhs, half, 1.0, V0, h->ldv, d0, ldw, 0.0, RHS + r, S_size);
  orc_dgemm('t', 'n', r, nrhs, half, 1.0, V1, h->ldv, d1, ldw, 0.0, RHS, S_size);
  if (s) {
    /* scale rows of the off-diagonal blocks and of the right-hand side */
    for (int j = 0; j < r; ++j)
      for (int i = 0; i < r; ++i) {
        S[(r + i) + (int64_t)j * S_size] *= s[i];
        S[i + (int64_t)(r + j) * S_size] *= s[i];
      }
    for (int j = 0; j < nrhs; ++j)
      for (int i = 0; i < r; ++i) {
        RHS[i + (int64_t)j * S_size] *= s[i];
        RHS[r + i + (int64_t)j * S_size] *= s[i];
      }
  }
  info = orc_dgetrf(S_size, S_size, S, S_size, ipiv);
  if (info == 0) {
    orc_dgetrs('N', S_size, nrhs, S, S_size, ipiv, RHS, S_size);
    orc_dgemm('n', 'n', half, nrhs, r, -1.0, u0, ldw, RHS, S_size, 1.0, d0, ldw);
    orc_dgemm('n', 'n', half, nrhs, r, -1.0, u1, ldw, RHS + r, S_size, 1.0, d1, ldw);
    int64_t node = ((int64_t)1 << depth) - 1 + pos;
    if (h->cap_lu)
      memcpy(h->cap_lu + node * S_size * S_size, S, sizeof(double) * S_size * S_size);
    if (h->cap_ipiv) memcpy(h->cap_ipiv + node * S_size, ipiv, sizeof(int) * S_size);
  } else {
    info = -(int)(((int64_t)1 << depth) - 1 + pos) - 1; /* -(node+1) */
  }
  free(S);
  free(RHS);
  free(ipiv);
  return info;
}

/* Returns 0; k>0 if leaf k-1 is singular; -(node+1) if a capacitance
 * system is singular. */
ORC_API int orc_hsolve_general(int leaf, int levels, int rank, double *K,
                               int64_t ldk, const double *const *V,
                               int64_t ldv, const double *const *s, int nrhs,
                               double *W, int64_t ldw, int *leaf_ipiv,
                               double *cap_lu, int *cap_ipiv) {
  orc_hodlr h = {leaf, levels, rank, K, ldk, V, ldv, s, leaf_ipiv, cap_lu, cap_ipiv};
  int64_t n = (int64_t)leaf << levels;
  return orc_hgen_rec(&h, 0, 0, (int)n, nrhs, W, ldw, 0);
}

/* ------------------------------------------------------------------------ */
/* Thread-parallel hsolve for the CPU baseline: the 2^p subtrees under       */
/* depth p run concurrently (one per thread, as the reference's index launch */
/* of LeafSolveTask over 2^launchlvl colours does, src/lmatrix.cc:449-493),  */
/* then depths p-1..0 run level by level with the row-chunked reduce /       */
/* capacitance / broadcast steps of GemmRed, NodeSolve and GemmBro          */
/* (src/tasks/gemm_reduce.cc:33-83, node_solve.cc:37-82,                     */
/* gemm_broadcast.cc:33-83).                                                 */
/* ------------------------------------------------------------------------ */
typedef struct {
  const orc_hodlr *h;
  int depth, nrow, nrhs, first, count, result;
  int64_t row0_base;
  double *W;
  int64_t ldw;
} orc_sub_job;

static void *orc_sub_worker(void *arg) {
  orc_sub_job *j = (orc_sub_job *)arg;
  j->result = 0;
  for (int q = j->first; q < j->first + j->count; ++q) {
    int info = orc_hgen_rec(j->h, j->depth, (int64_t)q * j->nrow, j->nrow,
                            j->nrhs, j->W, j->ldw, q);
    if (info && !j->result) j->result = info;
  }
  return NULL;
}

typedef struct {
  const double *V;
  const double *X;
  int64_t ldv, ldx;
  int64_t row0;
  int rows, r, ncol;
  double *out; /* r x ncol */
} orc_red_job;

static void *orc_red_worker(void *arg) {
  orc_red_job *j = (orc_red_job *)arg;
  orc_dgemm('t', 'n', j->r, j->ncol, j->rows, 1.0, j->V + j->row0, j->ldv,
            j->X + j->row0, j->ldx, 0.0, j->out, j->r);
  return NULL;
}

typedef struct {
  const double *u;
  const double *eta;
  double *d;
  int64_t ldw, row0;
  int rows, r, ncol, ldeta;
} orc_upd_job;

static void *orc_upd_worker(void *arg) {
  orc_upd_job *j = (orc_upd_job *)arg;
  orc_dgemm('n', 'n', j->rows, j->ncol, j->r, -1.0, j->u + j->row0, j->ldw,
            j->eta, j->ldeta, 1.0, j->d + j->row0, j->ldw);
  return NULL;
}

ORC_API int orc_hsolve_general_mt(int leaf, int levels, int rank, double *K,
                                  int64_t ldk, const double *const *V,
                                  int64_t ldv, const double *const *s,
                                  int nrhs, double *W, int64_t ldw,
                                  int nthreads) {
  orc_hodlr h = {leaf, levels, rank, K, ldk, V, ldv, s, NULL, NULL, NULL};
  int p = 0;
  while ((1 << (p + 1)) <= nthreads && p + 1 <= levels) ++p;
  int P = 1 << p;
  int64_t n = (int64_t)leaf << levels;
  int sub_rows = (int)(n >> p);
  const int r = rank;
  /* subtrees rooted at depth p */
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * P);
  orc_sub_job *jobs = (orc_sub_job *)malloc(sizeof(orc_sub_job) * P);
  for (int t = 0; t < P; ++t) {
    jobs[t] = (orc_sub_job){&h, p, sub_rows, nrhs + p * r, t, 1, 0, 0, W, ldw};
    pthread_create(&th[t], NULL, orc_sub_worker, &jobs[t]);
  }
  int info = 0;
  for (int t = 0; t < P; ++t) {
    pthread_join(th[t], NULL);
    if (jobs[t].result && !info) info = jobs[t].result;
  }
  free(jobs);
  if (info) {
    free(th);
    return info;
  }
  /* top levels, row-chunked across the P threads */
  orc_red_job *rj = (orc_red_job *)malloc(sizeof(orc_red_job) * P);
  orc_upd_job *uj = (orc_upd_job *)malloc(sizeof(orc_upd_job) * P);
  for (int depth = p - 1; depth >= 0; --depth) {
    int nodes = 1 << depth;
    int node_rows = (int)(n >> depth);
    int half = node_rows / 2;
    int dcols = nrhs + depth * r; /* columns of d at this depth */
    int ncol = dcols + r;         /* [d | u] */
    int S_size = 2 * r;
    int chunks_per_child = P / (2 * nodes);
    if (chunks_per_child < 1) chunks_per_child = 1;
    int chunk_rows = half / chunks_per_child;
    double *part = (double *)malloc(sizeof(double) * (size_t)P * r * ncol);
    for (int nd = 0; nd < nodes; ++nd) {
      int64_t row0 = (int64_t)nd * node_rows;
      double *T[2];
      for (int c = 0; c < 2; ++c) {
        T[c] = (double *)calloc((size_t)r * ncol, sizeof(double));
        int nj = 0;
        for (int q = 0; q < chunks_per_child; ++q, ++nj) {
          int rows = (q == chunks_per_child - 1) ? half - q * chunk_rows : chunk_rows;
          rj[nj] = (orc_red_job){V[depth], W, ldv, ldw, row0 + c * half + (int64_t)q * chunk_rows,
                                 rows, r, ncol, part + (size_t)nj * r * ncol};
          pthread_create(&th[nj], NULL, orc_red_worker, &rj[nj]);
        }
        for (int q = 0; q < nj; ++q) pthread_join(th[q], NULL);
        for (int q = 0; q < nj; ++q) /* Add reduction, in colour order */
          for (int e = 0; e < r * ncol; ++e) T[c][e] += part[(size_t)q * r * ncol + e];
      }
      /* NodeSolve: S = [I, s.V1'u1; s.V0'u0, I], RHS = [s.V1'd1; s.V0'd0] */
      double *S = (double *)calloc((size_t)S_size * S_size, sizeof(double));
      double *RHS = (double *)malloc(sizeof(double) * S_size * (dcols > 0 ? dcols : 1));
      int *ipiv = (int *)malloc(sizeof(int) * S_size);
      const double *sv = s ? s[depth] : NULL;
      for (int i = 0; i < S_size; ++i) S[i + (int64_t)i * S_size] = 1.0;
      for (int j = 0; j < r; ++j)
        for (int i = 0; i < r; ++i) {
          double sc = sv ? sv[i] : 1.0;
          S[(r + i) + (int64_t)j * S_size] = sc * T[0][i + (int64_t)(dcols + j) * r];
          S[i + (int64_t)(r + j) * S_size] = sc * T[1][i + (int64_t)(dcols + j) * r];
        }
      for (int j = 0; j < dcols; ++j)
        for (int i = 0; i < r; ++i) {
          double sc = sv ? sv[i] : 1.0;
          RHS[i + (int64_t)j * S_size] = sc * T[1][i + (int64_t)j * r];
          RHS[r + i + (int64_t)j * S_size] = sc * T[0][i + (int64_t)j * r];
        }
      int sinfo = orc_dgesv(S_size, dcols, S, S_size, ipiv, RHS, S_size);
      if (sinfo && !info) info = -(int)(((int64_t)1 << depth) - 1 + nd) - 1;
      /* GemmBro: d_c -= u_c eta_c, row-chunked */
      int nj = 0;
      for (int c = 0; c < 2 && !sinfo; ++c)
        for (int q = 0; q < chunks_per_child; ++q, ++nj) {
          int rows = (q == chunks_per_child - 1) ? half - q * chunk_rows : chunk_rows;
          uj[nj] = (orc_upd_job){W + (int64_t)dcols * ldw, RHS + (c == 0 ? 0 : r), W, ldw,
                                 row0 + c * half + (int64_t)q * chunk_rows, rows, r, dcols, S_size};
          pthread_create(&th[nj], NULL, orc_upd_worker, &uj[nj]);
        }
      for (int q = 0; q < nj; ++q) pthread_join(th[q], NULL);
      free(S);
      free(RHS);
      free(ipiv);
      free(T[0]);
      free(T[1]);
    }
    free(part);
  }
  free(rj);
  free(uj);
  free(th);
  return info;
}

/* ------------------------------------------------------------------------ */
/* FP64 HODLR matvec Y = A X from the exact representation (the residual     */
/* formula of tests/test.cc:654, generalised to per-level factors).          */
/* Dl: stacked leaf blocks (N x m, ld ldk); U[l], V[l]: N x r.               */
/* ------------------------------------------------------------------------ */
ORC_API void orc_hodlr_matvec(int leaf, int levels, int rank, const double *K,
                              int64_t ldk, const double *const *U,
                              int64_t ldu, const double *const *V,
                              int64_t ldv, const double *const *s, int nrhs,
                              const double *X, int64_t ldx, double *Y,
                              int64_t ldy) {
  int64_t n = (int64_t)leaf << levels;
  int nleaf = 1 << levels;
  for (int b = 0; b < nleaf; ++b)
    orc_dgemm('n', 'n', leaf, nrhs, leaf, 1.0, K + (int64_t)b * leaf, ldk,
              X + (int64_t)b * leaf, ldx, 0.0, Y + (int64_t)b * leaf, ldy);
  double *T = (double *)malloc(sizeof(double) * rank * (nrhs > 0 ? nrhs : 1));
  for (int l = 0; l < levels; ++l) {
    int64_t half = n >> (l + 1);
    for (int64_t c = 0; c < ((int64_t)2 << l); ++c) {
      int64_t src = c ^ 1; /* sibling supplies V^T x */
      orc_dgemm('t', 'n', rank, nrhs, (int)half, 1.0, V[l] + src * half, ldv,
                X + src * half, ldx, 0.0, T, rank);
      if (s && s[l])
        for (int j = 0; j < nrhs; ++j)
          for (int i = 0; i < rank; ++i) T[i + (int64_t)j * rank] *= s[l][i];
      orc_dgemm('n', 'n', (int)half, nrhs, rank, 1.0, U[l] + c * half, ldu, T,
                rank, 1.0, Y + c * half, ldy);
    }
  }
  free(T);
}
