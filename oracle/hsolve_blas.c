/*
 * hsolve_blas.c -- TEST INFRASTRUCTURE ONLY (the CPU baseline and the
 * full-size host checker).
 *
 * fastSolver2's HODLR solve hsolve (src/tasks/leaf_solve.cc:73-154) restated
 * with the BLAS/LAPACK calls it makes -- dgemm_ and dgesv_ with the same
 * shapes, leading dimensions and order -- routed to an optimised BLAS that
 * the caller names at run time (scipy's bundled OpenBLAS; its routines carry
 * a "scipy_" prefix).  Where the reference's own hsolve is compiled against
 * the same BLAS, hb_hsolve gives the same bits (tests/test_oracle.py).
 *
 * hb_hsolve_mt is the multi-core baseline the reference's Legion launch
 * amounts to on one node: the 2^p subtrees under depth p are solved
 * concurrently, one per thread (the LeafSolveTask index launch over 2^p
 * colours, src/lmatrix.cc:449-493), then depths p-1..0 run level by level as
 * row-chunked reductions V^T [d | u] (GemmRedTask, src/tasks/gemm_reduce.cc:
 * 33-83, partial blocks added in colour order as ReduceAdd does,
 * src/tasks/reduce_add.cc:7-49), one capacitance dgesv per node (NodeSolveTask,
 * src/tasks/node_solve.cc:37-82) and row-chunked updates d -= u eta
 * (GemmBroTask, src/tasks/gemm_broadcast.cc:33-83).  The BLAS runs single
 * threaded (the reference requires it, spmd_driver/Makefile:44-49); the
 * threads are ours.
 *
 * hb_matvec_mt is the FP64 HODLR product Y = A X from the exact
 * representation (the residual formula of tests/test.cc:654, per-level
 * factors), threaded over row ranges, for full-size residual checks.
 *
 * Column-major storage with explicit leading dimensions throughout
 * (src/ptr_matrix.cc:29-37).
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define HB_API __attribute__((visibility("default")))

typedef void (*dgemm_fn)(const char *, const char *, const int *, const int *, const int *, const double *,
                         const double *, const int *, const double *, const int *, const double *, double *,
                         const int *);
typedef void (*dgesv_fn)(const int *, const int *, double *, const int *, int *, double *, const int *, int *);
typedef void (*nthreads_fn)(int);

static dgemm_fn g_dgemm = NULL;
static dgesv_fn g_dgesv = NULL;

/* Bind the BLAS in the shared library at `path` (dlopen'ed; the scipy_ and
 * unprefixed names are both tried) and set its own threading to one thread.
 * Returns 0, or -1 if the library or a routine is missing. */
HB_API int hb_init(const char *path) {
  void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return -1;
  g_dgemm = (dgemm_fn)dlsym(h, "scipy_dgemm_");
  if (!g_dgemm) g_dgemm = (dgemm_fn)dlsym(h, "dgemm_");
  g_dgesv = (dgesv_fn)dlsym(h, "scipy_dgesv_");
  if (!g_dgesv) g_dgesv = (dgesv_fn)dlsym(h, "dgesv_");
  nthreads_fn set = (nthreads_fn)dlsym(h, "scipy_openblas_set_num_threads");
  if (!set) set = (nthreads_fn)dlsym(h, "openblas_set_num_threads");
  if (set) set(1);
  return (g_dgemm && g_dgesv) ? 0 : -1;
}

static void gemm(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda, const double *B,
                 int ldb, double beta, double *C, int ldc) {
  g_dgemm(&ta, &tb, &m, &n, &k, &alpha, A, &lda, B, &ldb, &beta, C, &ldc);
}

static int gesv(int n, int nrhs, double *A, int lda, int *ipiv, double *B, int ldb) {
  int info = 0;
  g_dgesv(&n, &nrhs, A, &lda, ipiv, B, &ldb, &info);
  return info;
}

/* ------------------------------------------------------------------------ */
/* hsolve (src/tasks/leaf_solve.cc:73-154): one V for every level, the U     */
/* chunks in the same region as the right-hand side.  Returns 0, the INFO    */
/* of a failing leaf dgesv, or -1000 - INFO for a capacitance system.        */
/* ------------------------------------------------------------------------ */
HB_API int hb_hsolve(int nrow, int nrhs, int rank, int nPart, int LD, double *K, double *U, double *V) {
  if (nPart == 1) {
    int *ipiv = (int *)malloc(sizeof(int) * (nrow > 0 ? nrow : 1));
    int info = gesv(nrow, nrhs, K, LD, ipiv, U, LD);
    free(ipiv);
    return info;
  }
  const int h = nrow / 2;
  double *d0 = U, *d1 = U + h;
  double *V0 = V, *V1 = V + h;
  double *u0 = d0 + (int64_t)nrhs * LD, *u1 = d1 + (int64_t)nrhs * LD;
  int info = hb_hsolve(h, nrhs + rank, rank, nPart / 2, LD, K, d0, V0);
  if (info) return info;
  info = hb_hsolve(h, nrhs + rank, rank, nPart / 2, LD, K + h, d1, V1);
  if (info) return info;
  const int S_size = 2 * rank;
  double *S = (double *)calloc((size_t)S_size * S_size, sizeof(double));
  double *RHS = (double *)malloc(sizeof(double) * S_size * (nrhs > 0 ? nrhs : 1));
  int *ipiv = (int *)malloc(sizeof(int) * S_size);
  for (int i = 0; i < S_size; ++i) S[S_size * i + i] = 1.0;
  /* S = [I, V1'u1; V0'u0, I] and RHS = [V1'd1; V0'd0] (swapped halves) */
  gemm('t', 'n', rank, rank, h, 1.0, V0, LD, u0, LD, 0.0, S + S_size / 2, S_size);
  gemm('t', 'n', rank, rank, h, 1.0, V1, LD, u1, LD, 0.0, S + S_size / 2 * S_size, S_size);
  gemm('t', 'n', rank, nrhs, h, 1.0, V0, LD, d0, LD, 0.0, RHS + S_size / 2, S_size);
  gemm('t', 'n', rank, nrhs, h, 1.0, V1, LD, d1, LD, 0.0, RHS, S_size);
  info = gesv(S_size, nrhs, S, S_size, ipiv, RHS, S_size);
  if (info == 0) {
    gemm('n', 'n', h, nrhs, rank, -1.0, u0, LD, RHS, S_size, 1.0, d0, LD);          /* eta0: top half */
    gemm('n', 'n', h, nrhs, rank, -1.0, u1, LD, RHS + S_size / 2, S_size, 1.0, d1, LD); /* eta1 */
  } else {
    info = -1000 - info;
  }
  free(S);
  free(RHS);
  free(ipiv);
  return info;
}

/* ------------------------------------------------------------------------ */
/* Per-level V^(l) (N x r, ld ldv): the node at depth l couples its children */
/* through A[c0,c1] = U^(l)_c0 V^(l)_c1^T, A[c1,c0] = U^(l)_c1 V^(l)_c0^T.   */
/* W (ld ldw) holds [B | U^(0) | ... | U^(L-1)] on entry and               */
/* [X | Utilde^(0) | ...] on exit, as hsolve leaves the UTree region.  With  */
/* every V[l] the same array this is hsolve.                                 */
/* ------------------------------------------------------------------------ */
typedef struct {
  int leaf, levels, rank;
  double *K;
  int ldk;
  const double *const *V;
  int ldv;
  double *W;
  int ldw;
} hb_tree;

static int hb_rec(const hb_tree *t, int depth, int64_t row0, int nrow, int nrhs) {
  const int r = t->rank;
  if (depth == t->levels) {
    int *ipiv = (int *)malloc(sizeof(int) * nrow);
    int info = gesv(nrow, nrhs, t->K + row0, t->ldk, ipiv, t->W + row0, t->ldw);
    free(ipiv);
    return info ? 1 : 0;
  }
  const int h = nrow / 2;
  int info = hb_rec(t, depth + 1, row0, h, nrhs + r);
  if (info) return info;
  info = hb_rec(t, depth + 1, row0 + h, h, nrhs + r);
  if (info) return info;
  const double *V0 = t->V[depth] + row0, *V1 = V0 + h;
  double *d0 = t->W + row0, *d1 = d0 + h;
  double *u0 = d0 + (int64_t)nrhs * t->ldw, *u1 = d1 + (int64_t)nrhs * t->ldw;
  const int S_size = 2 * r;
  double *S = (double *)calloc((size_t)S_size * S_size, sizeof(double));
  double *RHS = (double *)malloc(sizeof(double) * S_size * (nrhs > 0 ? nrhs : 1));
  int *ipiv = (int *)malloc(sizeof(int) * S_size);
  for (int i = 0; i < S_size; ++i) S[S_size * i + i] = 1.0;
  gemm('t', 'n', r, r, h, 1.0, V0, t->ldv, u0, t->ldw, 0.0, S + r, S_size);
  gemm('t', 'n', r, r, h, 1.0, V1, t->ldv, u1, t->ldw, 0.0, S + (int64_t)r * S_size, S_size);
  gemm('t', 'n', r, nrhs, h, 1.0, V0, t->ldv, d0, t->ldw, 0.0, RHS + r, S_size);
  gemm('t', 'n', r, nrhs, h, 1.0, V1, t->ldv, d1, t->ldw, 0.0, RHS, S_size);
  info = gesv(S_size, nrhs, S, S_size, ipiv, RHS, S_size);
  if (info == 0) {
    gemm('n', 'n', h, nrhs, r, -1.0, u0, t->ldw, RHS, S_size, 1.0, d0, t->ldw);
    gemm('n', 'n', h, nrhs, r, -1.0, u1, t->ldw, RHS + r, S_size, 1.0, d1, t->ldw);
  } else {
    info = 2;
  }
  free(S);
  free(RHS);
  free(ipiv);
  return info;
}

/* ------------------------------------------------------------------ threads */
typedef struct {
  void (*fn)(void *);
  void *arg;
} hb_job;

static void *hb_thread_main(void *p) {
  hb_job *j = (hb_job *)p;
  j->fn(j->arg);
  return NULL;
}

/* Run fn(args + i * stride) for i < n, one thread each, and join them. */
static void hb_parallel(int n, void (*fn)(void *), void *args, size_t stride) {
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * n);
  hb_job *jobs = (hb_job *)malloc(sizeof(hb_job) * n);
  for (int i = 0; i < n; ++i) {
    jobs[i].fn = fn;
    jobs[i].arg = (char *)args + (size_t)i * stride;
    pthread_create(&th[i], NULL, hb_thread_main, &jobs[i]);
  }
  for (int i = 0; i < n; ++i) pthread_join(th[i], NULL);
  free(jobs);
  free(th);
}

typedef struct {
  const hb_tree *t;
  int depth, nrow, nrhs, result;
  int64_t row0;
} hb_sub;

static void hb_sub_run(void *p) {
  hb_sub *s = (hb_sub *)p;
  s->result = hb_rec(s->t, s->depth, s->row0, s->nrow, s->nrhs);
}

typedef struct {
  const double *A; /* reduce: V rows; update: u rows */
  const double *B; /* reduce: [d | u] rows; update: eta */
  double *C;       /* reduce: partial r x ncol; update: d rows */
  int rows, r, ncol, lda, ldb, ldc;
} hb_gemm_job;

static void hb_reduce_run(void *p) {
  hb_gemm_job *j = (hb_gemm_job *)p;
  gemm('t', 'n', j->r, j->ncol, j->rows, 1.0, j->A, j->lda, j->B, j->ldb, 0.0, j->C, j->ldc);
}

static void hb_update_run(void *p) {
  hb_gemm_job *j = (hb_gemm_job *)p;
  gemm('n', 'n', j->rows, j->ncol, j->r, -1.0, j->A, j->lda, j->B, j->ldb, 1.0, j->C, j->ldc);
}

/* The threaded solve described in the header comment.  nthreads is rounded
 * down to a power of two P = 2^p (p <= levels).  Returns 0, 1 (a singular
 * leaf) or 2 (a singular capacitance system). */
HB_API int hb_hsolve_mt(int leaf, int levels, int rank, double *K, int64_t ldk, const double *const *V,
                        int64_t ldv, int nrhs, double *W, int64_t ldw, int nthreads) {
  hb_tree t = {leaf, levels, rank, K, (int)ldk, V, (int)ldv, W, (int)ldw};
  int p = 0;
  while ((1 << (p + 1)) <= nthreads && p + 1 <= levels) ++p;
  const int P = 1 << p, r = rank;
  const int64_t n = (int64_t)leaf << levels;
  const int sub_rows = (int)(n >> p);
  hb_sub *subs = (hb_sub *)malloc(sizeof(hb_sub) * P);
  for (int i = 0; i < P; ++i) subs[i] = (hb_sub){&t, p, sub_rows, nrhs + p * r, 0, (int64_t)i * sub_rows};
  hb_parallel(P, hb_sub_run, subs, sizeof(hb_sub));
  int info = 0;
  for (int i = 0; i < P && !info; ++i) info = subs[i].result;
  free(subs);
  if (info) return info;

  hb_gemm_job *jobs = (hb_gemm_job *)malloc(sizeof(hb_gemm_job) * P);
  const int S_size = 2 * r;
  for (int depth = p - 1; depth >= 0 && !info; --depth) {
    const int nodes = 1 << depth;
    const int node_rows = (int)(n >> depth), half = node_rows / 2;
    const int dcols = nrhs + depth * r, ncol = dcols + r; /* [d | u] */
    const int chunks = P / (2 * nodes);                  /* per child */
    const int chunk_rows = half / chunks;
    double *part = (double *)malloc(sizeof(double) * (size_t)P * r * ncol);
    /* GemmRed: every (node, child, chunk) at once */
    for (int j = 0; j < P; ++j) {
      const int64_t row = (int64_t)j * chunk_rows;
      jobs[j] = (hb_gemm_job){V[depth] + row, W + row, part + (size_t)j * r * ncol, chunk_rows, r, ncol,
                              (int)ldv, (int)ldw, r};
    }
    hb_parallel(P, hb_reduce_run, jobs, sizeof(hb_gemm_job));
    /* ReduceAdd in colour order, then NodeSolve per node */
    double *eta = (double *)malloc(sizeof(double) * (size_t)nodes * S_size * (dcols > 0 ? dcols : 1));
    double *T = (double *)malloc(sizeof(double) * 2 * (size_t)r * ncol);
    double *S = (double *)malloc(sizeof(double) * S_size * S_size);
    int *ipiv = (int *)malloc(sizeof(int) * S_size);
    for (int nd = 0; nd < nodes && !info; ++nd) {
      for (int c = 0; c < 2; ++c) {
        double *Tc = T + (size_t)c * r * ncol;
        const double *first = part + (size_t)((2 * nd + c) * chunks) * r * ncol;
        memcpy(Tc, first, sizeof(double) * r * ncol);
        for (int q = 1; q < chunks; ++q) {
          const double *pq = first + (size_t)q * r * ncol;
          for (int e = 0; e < r * ncol; ++e) Tc[e] += pq[e];
        }
      }
      double *RHS = eta + (size_t)nd * S_size * dcols;
      memset(S, 0, sizeof(double) * S_size * S_size);
      for (int i = 0; i < S_size; ++i) S[i + i * S_size] = 1.0;
      for (int j = 0; j < r; ++j)
        for (int i = 0; i < r; ++i) {
          S[(r + i) + j * S_size] = T[i + (int64_t)(dcols + j) * r];                            /* V0'u0 */
          S[i + (r + j) * S_size] = T[(size_t)r * ncol + i + (int64_t)(dcols + j) * r];         /* V1'u1 */
        }
      for (int j = 0; j < dcols; ++j)
        for (int i = 0; i < r; ++i) {
          RHS[i + (int64_t)j * S_size] = T[(size_t)r * ncol + i + (int64_t)j * r];  /* V1'd1 */
          RHS[r + i + (int64_t)j * S_size] = T[i + (int64_t)j * r];                 /* V0'd0 */
        }
      if (gesv(S_size, dcols, S, S_size, ipiv, RHS, S_size)) info = 2;
    }
    /* GemmBro: d_c -= u_c eta_c, every chunk at once */
    if (!info) {
      for (int j = 0; j < P; ++j) {
        const int nd = j / (2 * chunks), c = (j / chunks) & 1;
        const int64_t row = (int64_t)j * chunk_rows;
        jobs[j] = (hb_gemm_job){W + (int64_t)dcols * ldw + row, eta + (size_t)nd * S_size * dcols + c * r,
                                W + row, chunk_rows, r, dcols, (int)ldw, S_size, (int)ldw};
      }
      hb_parallel(P, hb_update_run, jobs, sizeof(hb_gemm_job));
    }
    free(part);
    free(eta);
    free(T);
    free(S);
    free(ipiv);
  }
  free(jobs);
  return info;
}

/* ------------------------------------------------------------------------ */
/* Y = A X from the exact representation: leaf blocks K (N x m stacked, ld   */
/* ldk), U[l], V[l] (N x r, ld ldu / ldv), optional s[l] (r entries; the      */
/* coupling is U diag(s) V^T).  Rows split into P = 2^p ranges, one thread   */
/* each: first every (range, child block) partial V^T X, summed per block in */
/* range order, then each thread forms its own rows of Y.                    */
/* ------------------------------------------------------------------------ */
typedef struct {
  int leaf, levels, rank, nrhs;
  const double *K;
  int ldk;
  const double *const *U;
  int ldu;
  const double *const *V;
  int ldv;
  const double *const *s;
  const double *X;
  int ldx;
  double *Y;
  int ldy;
  int64_t n;
  int P;
  double **T;    /* T[l]: 2^(l+1) blocks of r x nrhs (after summing: V_c^T X_c) */
  double **part; /* part[l]: per block, one r x nrhs partial per row range meeting it */
} hb_mv;

/* Row ranges (of n / P rows) that meet one child block at level l. */
static int64_t hb_slots(const hb_mv *m, int l) {
  const int64_t bs = m->n >> (l + 1), rows_per = m->n / m->P;
  return bs > rows_per ? bs / rows_per : 1;
}

typedef struct {
  hb_mv *m;
  int tid;
} hb_mv_arg;

static void hb_mv_reduce(void *p) {
  hb_mv_arg *a = (hb_mv_arg *)p;
  hb_mv *m = a->m;
  const int64_t lo = a->tid * (m->n / m->P), hi = lo + m->n / m->P;
  const int r = m->rank, k = m->nrhs;
  for (int l = 0; l < m->levels; ++l) {
    const int64_t bs = m->n >> (l + 1);
    const int64_t nb = (int64_t)2 << l;
    for (int64_t c = lo / bs; c < nb && c * bs < hi; ++c) {
      int64_t a0 = c * bs > lo ? c * bs : lo, a1 = (c + 1) * bs < hi ? (c + 1) * bs : hi;
      /* partial slot: block c, range a->tid (ranges that meet block c are consecutive) */
      const int64_t first = (c * bs) / (m->n / m->P);
      double *dst = m->part[l] + ((size_t)c * hb_slots(m, l) + (a->tid - first)) * r * k;
      gemm('t', 'n', r, k, (int)(a1 - a0), 1.0, m->V[l] + a0, m->ldv, m->X + a0, m->ldx, 0.0, dst, r);
    }
  }
}

static void hb_mv_apply(void *p) {
  hb_mv_arg *a = (hb_mv_arg *)p;
  hb_mv *m = a->m;
  const int64_t lo = a->tid * (m->n / m->P), hi = lo + m->n / m->P;
  const int r = m->rank, k = m->nrhs, mm = m->leaf;
  for (int64_t b = lo / mm; b * mm < hi; ++b)
    gemm('n', 'n', mm, k, mm, 1.0, m->K + b * mm, m->ldk, m->X + b * mm, m->ldx, 0.0, m->Y + b * mm, m->ldy);
  for (int l = 0; l < m->levels; ++l) {
    const int64_t bs = m->n >> (l + 1);
    const int64_t nb = (int64_t)2 << l;
    for (int64_t c = lo / bs; c < nb && c * bs < hi; ++c) {
      int64_t a0 = c * bs > lo ? c * bs : lo, a1 = (c + 1) * bs < hi ? (c + 1) * bs : hi;
      const double *Tsib = m->T[l] + (size_t)(c ^ 1) * r * k;
      gemm('n', 'n', (int)(a1 - a0), k, r, 1.0, m->U[l] + a0, m->ldu, Tsib, r, 1.0, m->Y + a0, m->ldy);
    }
  }
}

HB_API void hb_matvec_mt(int leaf, int levels, int rank, const double *K, int64_t ldk, const double *const *U,
                         int64_t ldu, const double *const *V, int64_t ldv, const double *const *s, int nrhs,
                         const double *X, int64_t ldx, double *Y, int64_t ldy, int nthreads) {
  const int64_t n = (int64_t)leaf << levels;
  int p = 0;
  while ((1 << (p + 1)) <= nthreads && p + 1 <= levels) ++p;
  const int P = 1 << p, r = rank, k = nrhs;
  hb_mv m = {leaf, levels, rank, nrhs, K, (int)ldk, U, (int)ldu, V, (int)ldv, s, X, (int)ldx, Y, (int)ldy, n, P,
             NULL, NULL};
  m.T = (double **)calloc(levels > 0 ? levels : 1, sizeof(double *));
  m.part = (double **)calloc(levels > 0 ? levels : 1, sizeof(double *));
  for (int l = 0; l < levels; ++l) {
    const size_t nb = (size_t)2 << l;
    m.T[l] = (double *)calloc(nb * r * k, sizeof(double));
    m.part[l] = (double *)calloc(nb * hb_slots(&m, l) * r * k, sizeof(double));
  }
  hb_mv_arg *args = (hb_mv_arg *)malloc(sizeof(hb_mv_arg) * P);
  for (int i = 0; i < P; ++i) args[i] = (hb_mv_arg){&m, i};
  hb_parallel(P, hb_mv_reduce, args, sizeof(hb_mv_arg));
  for (int l = 0; l < levels; ++l) {
    const int64_t bs = n >> (l + 1), nb = (int64_t)2 << l, rows_per = n / P;
    for (int64_t c = 0; c < nb; ++c) {
      const int64_t first = (c * bs) / rows_per, last = ((c + 1) * bs - 1) / rows_per;
      double *Tc = m.T[l] + (size_t)c * r * k;
      for (int64_t q = first; q <= last; ++q) {
        const double *src = m.part[l] + ((size_t)c * hb_slots(&m, l) + (q - first)) * r * k;
        for (int e = 0; e < r * k; ++e) Tc[e] += src[e];
      }
      if (s && s[l])
        for (int j = 0; j < k; ++j)
          for (int i = 0; i < r; ++i) Tc[i + (size_t)j * r] *= s[l][i];
    }
  }
  hb_parallel(P, hb_mv_apply, args, sizeof(hb_mv_arg));
  for (int l = 0; l < levels; ++l) {
    free(m.T[l]);
    free(m.part[l]);
  }
  free(m.T);
  free(m.part);
  free(args);
}

/* ------------------------------------------------------------------------ */
/* dst <- src, `bytes` bytes, split over nthreads threads (restoring the     */
/* in-place inputs between timed solves).                                    */
/* ------------------------------------------------------------------------ */
typedef struct {
  char *dst;
  const char *src;
  size_t bytes;
} hb_copy_job;

static void hb_copy_run(void *p) {
  hb_copy_job *j = (hb_copy_job *)p;
  memcpy(j->dst, j->src, j->bytes);
}

HB_API void hb_copy_mt(void *dst, const void *src, int64_t bytes, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  hb_copy_job *jobs = (hb_copy_job *)malloc(sizeof(hb_copy_job) * nthreads);
  const size_t step = ((size_t)bytes / nthreads + 4095) & ~(size_t)4095;
  int nj = 0;
  for (size_t off = 0; off < (size_t)bytes; off += step, ++nj) {
    const size_t len = off + step < (size_t)bytes ? step : (size_t)bytes - off;
    jobs[nj] = (hb_copy_job){(char *)dst + off, (const char *)src + off, len};
  }
  hb_parallel(nj, hb_copy_run, jobs, sizeof(hb_copy_job));
  free(jobs);
}

/* ------------------------------------------------------------------------ */
/* Seeded Gaussian fill for the baseline's inputs (a counter-based generator: */
/* element (i, j) of a rows x cols block draws from splitmix64 of            */
/* (seed, j * rows + i), two uniforms -> Box-Muller), times `scale`, plus    */
/* `diag` on the diagonal of every consecutive `diag_block` x `diag_block`   */
/* square (0 = none).  Columns split over nthreads threads.                 */
/* ------------------------------------------------------------------------ */
static uint64_t hb_mix(uint64_t z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

typedef struct {
  double *A;
  int64_t rows, lda, col0, col1, diag_block;
  uint64_t seed;
  double scale, diag;
} hb_fill_job;

static void hb_fill_run(void *p) {
  hb_fill_job *j = (hb_fill_job *)p;
  const double two_pi = 6.283185307179586476925286766559;
  for (int64_t c = j->col0; c < j->col1; ++c) {
    double *col = j->A + c * j->lda;
    for (int64_t i = 0; i < j->rows; ++i) {
      const uint64_t ctr = (uint64_t)(c * j->rows + i);
      const uint64_t a = hb_mix(j->seed ^ hb_mix(2 * ctr)), b = hb_mix(j->seed ^ hb_mix(2 * ctr + 1));
      const double u1 = ((double)(a >> 11) + 0.5) * (1.0 / 9007199254740992.0);
      const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
      double v = sqrt(-2.0 * log(u1)) * cos(two_pi * u2) * j->scale;
      if (j->diag_block > 0 && (i % j->diag_block) == c) v += j->diag;
      col[i] = v;
    }
  }
}

HB_API void hb_fill_gaussian(double *A, int64_t rows, int64_t cols, int64_t lda, uint64_t seed, double scale,
                             double diag, int64_t diag_block, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > cols) nthreads = (int)(cols > 0 ? cols : 1);
  hb_fill_job *jobs = (hb_fill_job *)malloc(sizeof(hb_fill_job) * nthreads);
  for (int t = 0; t < nthreads; ++t)
    jobs[t] = (hb_fill_job){A, rows, lda, cols * t / nthreads, cols * (t + 1) / nthreads, diag_block, seed,
                            scale, diag};
  hb_parallel(nthreads, hb_fill_run, jobs, sizeof(hb_fill_job));
  free(jobs);
}
