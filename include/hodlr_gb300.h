/*
 * hodlr_gb300.h -- C ABI of the GB300 HODLR (hierarchically off-diagonal
 * low-rank) fast direct solver.
 *
 * The matrix is A = blockdiag(D_leaf) + hierarchical off-diagonal low rank:
 * for a node p at depth l (root depth 0, leaves at depth L) with children
 * c0, c1,
 *     A[c0,c1] = U^(l)_c0 diag(s^(l)) V^(l)_c1^T,
 *     A[c1,c0] = U^(l)_c1 diag(s^(l)) V^(l)_c0^T,
 * where U^(l), V^(l) are N x r and X_c denotes the rows of child c.
 * fastSolver2 is the special case U^(l) = U, V^(l) = V, s = 1 for every l,
 * i.e. A = U V^T + diag(D) (src/tasks/dense_block.cc:63-75, tests/test.cc:654).
 *
 * Conventions (as in the reference, src/ptr_matrix.cc:29-37): FP64,
 * column-major, explicit leading dimensions.  Every entry point returns an
 * int status (HODLR_OK = 0); hodlr_last_error_string() describes the last
 * failure on the calling thread.  Calls on one handle are ordered on the
 * handle's CUDA stream; a handle is not thread-safe, distinct handles are.
 */
#ifndef HODLR_GB300_H
#define HODLR_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define HODLR_API __attribute__((visibility("default")))
#else
#define HODLR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  HODLR_OK = 0,
  HODLR_ERR_INVALID_ARG = 1,
  HODLR_ERR_CUDA = 2,
  HODLR_ERR_SINGULAR_LEAF = 3,          /* zero pivot in a leaf LU (index = leaf) */
  HODLR_ERR_SINGULAR_CAPACITANCE = 4,   /* zero pivot in a 2r x 2r system (index = node) */
  HODLR_ERR_NOT_CONVERGED = 5,          /* refinement hit its iteration cap */
  HODLR_ERR_NONFINITE_INPUT = 6,        /* NaN/Inf in an input (index = row) */
  HODLR_ERR_TIMEOUT = 7,                /* a bounded device wait expired */
  HODLR_ERR_NOT_FACTORED = 8,           /* solve before factor / inputs incomplete */
  HODLR_ERR_OUT_OF_MEMORY = 9
};

/* ------------------------------------------------------------- precision */
enum {
  HODLR_PREC_FP64 = 0,   /* every step in FP64 */
  HODLR_PREC_MIXED = 1   /* FP32 leaf LU / low-rank GEMMs, FP64 capacitance,
                            FP64-accurate residual + iterative refinement */
};

/* Residual arithmetic of the mixed path. */
enum {
  HODLR_RESID_FP64 = 0,          /* native FP64 (DFMA) */
  HODLR_RESID_FP64_EMULATED = 1, /* FP64-accurate double-FP32 arithmetic on
                                    the FP32 pipes (error-free products,
                                    double-word sums) */
  HODLR_RESID_FP64_TENSOR = 2    /* FP64-accurate products on the tensor cores:
                                    operands cut into exact 7-bit bf16 digits,
                                    exact FP32 digit-product sums, double-word
                                    combination (leaf sizes multiple of 64 up
                                    to 256, ranks multiple of 8 up to 64; other
                                    shapes and transposed solves use the
                                    double-word residual) */
};

/* hodlr_desc.flags */
enum {
  HODLR_FLAG_STREAM_INPUTS = 1  /* hodlr_set_lowrank with V in pinned host memory copies U at once and
                                   leaves V's copy to the next hodlr_factor, which streams the levels'
                                   V deepest first alongside the sweep (level l waits only for its own V):
                                   the host V buffers must stay valid until that hodlr_factor returns */
};

typedef struct hodlr_desc {
  int64_t n;              /* N = leaf * 2^levels */
  int32_t leaf;           /* m, leaf block size */
  int32_t levels;         /* L, tree depth (0 = one dense block) */
  int32_t rank;           /* r, off-diagonal rank (1..64) */
  int32_t nrhs_max;       /* largest nrhs a solve will be given */
  int32_t precision;      /* HODLR_PREC_* */
  int32_t residual;       /* HODLR_RESID_* (mixed path only) */
  double refine_tol;      /* target max_j ||b_j - A x_j|| / ||b_j|| (mixed), e.g. 1e-12 */
  int32_t refine_max_iter;/* refinement iteration cap (mixed) */
  int32_t flags;          /* HODLR_FLAG_* (0: none) */
  void *stream;           /* cudaStream_t; NULL = legacy default stream */
} hodlr_desc;

typedef struct hodlr_solve_info {
  int32_t iterations;     /* refinement corrections applied (0 for FP64) */
  int32_t status;         /* device status of the call (HODLR_*) */
  int64_t bad_index;      /* leaf / node / row named by a failing status */
  double rel_residual;    /* final max_j ||b_j - A x_j|| / ||b_j|| (mixed; -1 if not computed) */
} hodlr_solve_info;

typedef struct hodlr_ctx *hodlr_handle;

/* Gradients of a scalar loss through x = A^{-1} b, given g = dLoss/dx.
 * Device pointers; any may be NULL to skip it.  Layouts match the inputs:
 * dD like the leaf blocks set by hodlr_set_leaf_blocks (packed [leaf][m][m]
 * column-major), dU[l]/dV[l] N x r column-major with leading dimension n,
 * ds[l] r entries, db N x nrhs with leading dimension ldb. */
typedef struct hodlr_grads {
  double *db;  int64_t ldb;
  double *dD;
  double *dU;  /* L blocks of N x r, level l at dU + l*n*r */
  double *dV;  /* same layout */
  double *ds;  /* L blocks of r */
} hodlr_grads;

/* ------------------------------------------------- reference entry point */
/* Drop-in for fastSolver2's raw-pointer solve
 *   void hsolve(int nrow, int nrhs, int rank, int nPart, int LD,
 *               double *K, double *U, double *V)
 * (src/tasks/leaf_solve.cc:8-10, definition :73-154; called by
 * LeafSolveTask::cpu_task :69-70).  Same arguments, same in-place result:
 * K (nrow x nrow/nPart stacked leaf blocks, leading dimension LD) is
 * overwritten by the leaf LU factors (LAPACK dgesv layout), and U
 * (nrow x (nrhs + log2(nPart)*rank), leading dimension LD) goes from
 * [b | U ... U] to [x | Utilde^(0) | ... ], the way hsolve leaves it.
 * V (nrow x rank, leading dimension LD) is read only; it is shared by all
 * levels as in the reference.  Pointers may be host or device memory
 * (host buffers are staged through the device).  Runs on the legacy
 * default stream in FP64 and returns when the result is in place. */
HODLR_API int hodlr_hsolve(int nrow, int nrhs, int rank, int nPart, int LD, double *K,
                 double *U, double *V);

/* hodlr_hsolve with a precision mode and a stream (device pointers only
 * when stream is not NULL). */
HODLR_API int hodlr_hsolve_ex(int nrow, int nrhs, int rank, int nPart, int LD,
                    double *K, double *U, double *V, int precision,
                    void *stream, hodlr_solve_info *info);

/* ------------------------------------------- factor / solve handle API  */
/* Replaces HMatrix(nProc, level) + HMatrix::init(U, V, D) + the UTree /
 * VTree / KTree partitions (src/hmatrix.cc:7-47, src/tree.cc:42-245).      */
HODLR_API int hodlr_create(const hodlr_desc *desc, hodlr_handle *out);
HODLR_API int hodlr_destroy(hodlr_handle h);
HODLR_API int hodlr_set_stream(hodlr_handle h, void *stream);

/* Leaf blocks: leaf i's m x m block starts at D + i*leaf_stride, column-major
 * with leading dimension ld.  fastSolver2's KTree region (N x m, LD = N,
 * leaf i at rows i*m) is ld = N, leaf_stride = m
 * (src/tree.cc:232-245, src/tasks/dense_block.cc:63-75).  Device or host
 * pointer (pinned host memory is copied asynchronously on the stream). */
HODLR_API int hodlr_set_leaf_blocks(hodlr_handle h, const double *D, int64_t ld,
                          int64_t leaf_stride);

/* Low-rank factors of level l (0 = root split): U, V are N x r column-major
 * with leading dimensions ldu, ldv; s is r entries or NULL (= ones).
 * Replaces the UTree column chunk and VTree::level(i) (src/tree.cc:61-73,
 * 189-197).  Device or host pointers. */
HODLR_API int hodlr_set_lowrank(hodlr_handle h, int level, const double *U, int64_t ldu,
                      const double *V, int64_t ldv, const double *s);

/* The reference's HMatrix::init(U, V, D) (src/hmatrix.cc:22-47): A = U V^T +
 * diag(D) in HODLR form -- every level gets the same U and V (N x r,
 * leading dimensions ldu, ldv; VTree::level, src/tree.cc:189-197) and each
 * leaf block is U_i V_i^T + diag(D_i) (DenseBlockTask,
 * src/tasks/dense_block.cc:63-75).  D: N entries.  Host or device pointers. */
HODLR_API int hodlr_set_uvd(hodlr_handle h, const double *U, int64_t ldu, const double *V, int64_t ldv,
                            const double *D);

/* Factorisation: leaf LUs, transformed bases Utilde^(l) = A_c^{-1} U^(l)_c and
 * the 2r x 2r capacitance LUs of every node -- the work hsolve redoes on
 * every call with U as extra right-hand sides (src/tasks/leaf_solve.cc:80-153,
 * src/hmatrix.cc:75-93).  Returns after the device finished (status read). */
HODLR_API int hodlr_factor(hodlr_handle h);

/* Solve A X = B in place (B device, N x nrhs, leading dimension ldb).  In the
 * mixed mode this includes FP64 iterative refinement to desc.refine_tol.
 * Replaces HMatrix::solve (src/hmatrix.cc:49-96).  info may be NULL. */
HODLR_API int hodlr_solve(hodlr_handle h, double *B, int64_t ldb, int nrhs,
                hodlr_solve_info *info);

/* Solve A^T X = B in place, reusing the factorisation of A. */
HODLR_API int hodlr_solve_transpose(hodlr_handle h, double *B, int64_t ldb, int nrhs,
                          hodlr_solve_info *info);

/* Y = A X (or A^T X) in FP64 from the exact representation (device). */
HODLR_API int hodlr_matvec(hodlr_handle h, int transpose, const double *X, int64_t ldx,
                 double *Y, int64_t ldy, int nrhs);

/* Adjoint sweep: lambda = A^{-T} g, then db = lambda and the rank-nrhs outer
 * products dD_leaf = -lambda_i x_i^T, dU^(l), dV^(l), ds^(l) of
 * dLoss/dA = -lambda x^T.  x is the forward solution (N x nrhs, ldx),
 * g = dLoss/dx (N x nrhs, ldg).  Device pointers. */
HODLR_API int hodlr_adjoint(hodlr_handle h, const double *x, int64_t ldx,
                  const double *g, int64_t ldg, int nrhs, hodlr_grads *grads);

/* Copy out the factorisation (device pointers; any may be NULL):
 * leaf LU [nleaf][m][m] column-major + 1-based pivots [nleaf][m],
 * Utilde (N x L*r, leading dimension N, level l at column l*r),
 * capacitance LU [nnode][2r][2r] + pivots [nnode][2r] (node of depth l,
 * position p is 2^l - 1 + p).  FP64 handles only. */
HODLR_API int hodlr_get_factors(hodlr_handle h, double *leaf_lu, int32_t *leaf_ipiv,
                      double *utilde, double *cap_lu, int32_t *cap_ipiv);

/* The reference's seeded inputs, bit for bit (Matrix::rand src/matrix.cc:
 * 250-297, PtrMatrix::rand src/ptr_matrix.cc:62-71, the MapSeed argument maps
 * src/lmatrix.cc:327-360, DenseBlockTask src/tasks/dense_block.cc:35-76),
 * generated in device memory.  drand48 is the POSIX 48-bit LCG.
 * hodlr_draw_seeds: n per-partition seeds as Matrix::rand draws them
 * (srand48(master), then n lrand48 draws) into host memory; the reference
 * seeds `master` from the clock, a caller passes it.
 * hodlr_rand_matrix: A (device, column-major, lda >= npart*rows) gets npart
 * row partitions of `rows` rows; partition k is filled in row-major order
 * from the drand48 stream of seeds[k] (host array), each draw + offset.
 * Runs on `stream` (NULL = legacy default) and returns when done.
 * hodlr_set_seeded: the handle's inputs as HMatrix::init(U, V, D) builds them
 * from per-leaf seeds (host arrays of 2^levels): U and V (N x r, the same at
 * every level), D (N entries, draws + offset), leaf blocks U_k V_k^T +
 * diag(D_k) in the reference's BLAS order; s = 1. */
HODLR_API int hodlr_draw_seeds(int64_t master, int n, int64_t *seeds);
HODLR_API int hodlr_rand_matrix(const int64_t *seeds, int npart, int64_t rows, int cols, double offset, double *A,
                                int64_t lda, void *stream);
HODLR_API int hodlr_set_seeded(hodlr_handle h, const int64_t *useeds, const int64_t *vseeds, const int64_t *dseeds,
                               double offset);

/* Trees whose leaves have unequal sizes (the reference's
 * spmd_driver/solver_irregular_part.cc: subtrees with different leaf sizes)
 * embed exactly in the uniform tree: every leaf is padded to m_max rows with
 * an identity diagonal block, and the padded rows of U, V and of the
 * right-hand sides are zero.  After a permutation the padded matrix is
 * block diagonal in (real rows, padded rows), so its solution on the real
 * rows is the unequal-leaf system's and its padded rows stay zero.  Create
 * the handle with n = nleaf * m_max and leaf = m_max.
 * hodlr_pad_rows: rows of leaf i of src (packed: rows sz[0] + .. + sz[i-1]
 *   onwards, cols columns, leading dimension lds) to rows i * m_max .. of
 *   dst (leading dimension ldd), zeros in the padding.
 * hodlr_unpad_rows: the inverse, padded src to packed dst.
 * hodlr_pad_leaf_blocks: leaf blocks packed one after another (block i:
 *   sz[i] x sz[i], column-major) to [nleaf][m_max][m_max], ready for
 *   hodlr_set_leaf_blocks(h, dst, m_max, m_max * m_max).
 * sz: host array of nleaf sizes in [1, m_max]; src and dst device memory;
 * run on `stream` (NULL = legacy default) and return when done. */
HODLR_API int hodlr_pad_rows(int nleaf, const int32_t *sz, int m_max, int cols, const double *src, int64_t lds,
                             double *dst, int64_t ldd, void *stream);
HODLR_API int hodlr_unpad_rows(int nleaf, const int32_t *sz, int m_max, int cols, const double *src, int64_t lds,
                               double *dst, int64_t ldd, void *stream);
HODLR_API int hodlr_pad_leaf_blocks(int nleaf, const int32_t *sz, int m_max, const double *src, double *dst,
                                    void *stream);

/* Checkpoint of a factored plain handle (no counterpart in the reference,
 * which refactors on every solve): the descriptor, the launch shapes, the
 * inputs and every factor buffer in one host byte stream with a checksum.
 * hodlr_checkpoint_size gives the byte count; hodlr_checkpoint_save writes
 * it into host memory `buf` of `bytes` bytes; hodlr_checkpoint_load creates a
 * factored handle from it on `stream` (NULL = a stream of its own) whose
 * solves give the same bits as the saved handle's.  Batch handles have no
 * checkpoint (HODLR_ERR_INVALID_ARG); a corrupted or truncated stream is
 * refused with HODLR_ERR_INVALID_ARG. */
HODLR_API int hodlr_checkpoint_size(hodlr_handle h, int64_t *bytes);
HODLR_API int hodlr_checkpoint_save(hodlr_handle h, void *buf, int64_t bytes);
HODLR_API int hodlr_checkpoint_load(const void *buf, int64_t bytes, void *stream, hodlr_handle *out);

/* ------------------------------------------------- component entry points */
/* LMatrix::gemmRed('t', 'n', 1.0, V, U, 0.0, W) over nPart row partitions
 * (src/lmatrix.cc:713-761, GemmRedTask src/tasks/gemm_reduce.cc:33-83):
 * W rows [p*ncolV, (p+1)*ncolV) = V_p^T U_p, V_p / U_p the rows
 * [p*nrow/nPart, (p+1)*nrow/nPart) of V (nrow x ncolV) and U (nrow x ncolU).
 * ncolV <= 64.  Device pointers, column-major. */
HODLR_API int hodlr_gemm_reduce(int nrow, int nPart, int ncolV, int ncolU, const double *V, int64_t ldv,
                                const double *U, int64_t ldu, double *W, int64_t ldw);

/* hodlr_gemm_reduce for callers that may not allocate device memory
 * (frameworks that own the device through their own allocator, loops that
 * cannot absorb cudaMalloc's synchronisation).  No counterpart in the
 * reference.  Same arguments and result; its scratch is a fixed 16 MiB device
 * array inside the library (2^21 doubles, held on every GPU that loads the
 * library) instead of cudaMalloc.  nPart*ncolV*ncolU plus the split-K partial
 * sums must fit that array, else HODLR_ERR_INVALID_ARG.  The first call on a
 * device looks up the array's address and caches it (not valid after
 * cudaDeviceReset on that device); calls that overlap on the GPU share the
 * array and race.  Runs on the legacy default stream and returns when W is
 * written. */
HODLR_API int hodlr_gemm_reduce_noalloc(int nrow, int nPart, int ncolV, int ncolU, const double *V,
                                        int64_t ldv, const double *U, int64_t ldu, double *W, int64_t ldw);

/* LMatrix::gemmBro('n', 'n', alpha, U, Vb, beta, W) (src/lmatrix.cc:814-865,
 * GemmBroTask src/tasks/gemm_broadcast.cc:33-83): the nrow rows of U and W
 * split into nPart partitions, Vb into nBlock row blocks of K rows (nPart a
 * multiple of nBlock); partition p uses block p / (nPart / nBlock):
 * W_p = alpha U_p Vb_block + beta W_p.  Device pointers, column-major. */
HODLR_API int hodlr_gemm_broadcast(int nrow, int nPart, int nBlock, int K, int N, double alpha, const double *U,
                                   int64_t ldu, const double *Vb, int64_t ldvb, double beta, double *W,
                                   int64_t ldw);

/* LMatrix::node_solve / NodeSolveTask (src/lmatrix.cc:534-581,
 * src/tasks/node_solve.cc:37-82) for nnode nodes: node p's rows
 * [2r p, 2r (p+1)) of VTu hold [V0^T u0; V1^T u1] (2r x r) and of VTd
 * [V0^T d0; V1^T d1] (2r x nrhs).  S = [I, V1^T u1; V0^T u0, I] is solved
 * against the swapped right-hand side [V1^T d1; V0^T d0] and the solution
 * (eta0; eta1) overwrites VTd.  FP64 LU with partial pivoting.  Device
 * pointers, column-major. */
HODLR_API int hodlr_node_solve(int nnode, int r, int nrhs, const double *VTu, int64_t ldu, double *VTd,
                               int64_t ldd);

/* NodeSolveRegionTask (src/tasks/node_solve_region.cc:77-97) for nnode
 * nodes whose children have unequal ranks r0, r1 (1..64 each): node p's
 * blocks are rows [p r1, (p+1) r1) of VTu0 (V0^T u0, nnode r1 x r0) and VTd0
 * (nnode r1 x nrhs), rows [p r0, (p+1) r0) of VTu1 (V1^T u1, nnode r0 x r1)
 * and VTd1 (nnode r0 x nrhs).  S = [I_r0, VTu1; VTu0, I_r1] ((r0+r1)-square)
 * is solved against [VTd1; VTd0] by FP64 LU with partial pivoting, and the
 * solution is copied back as the reference does: its first r0 rows into
 * VTd1, the last r1 into VTd0.  Device pointers, column-major; synchronous. */
HODLR_API int hodlr_node_solve_irregular(int nnode, int r0, int r1, int nrhs, const double *VTu0, int64_t ldu0,
                                         const double *VTu1, int64_t ldu1, double *VTd0, int64_t ldd0,
                                         double *VTd1, int64_t ldd1);

/* Copy out the problem held by the handle (device or host destinations; any
 * may be NULL): leaf blocks in the layout of hodlr_set_leaf_blocks
 * (ld, leaf_stride), U and V as L blocks of N x r (leading dimension N,
 * level l at + l*N*r), s as L blocks of r. */
HODLR_API int hodlr_get_inputs(hodlr_handle h, double *D, int64_t ld, int64_t leaf_stride, double *U,
                               double *V, double *s);

/* Fill the handle with a seeded synthetic problem on the device
 * (counter-based Gaussian generator): leaf blocks G/sqrt(m) + shift*I,
 * per-level U, V ~ N(0,1)/sqrt(n_block) (orthonormal != 0: each child
 * block's columns orthonormalised instead), s_i = 10^(-decay*i/r) when
 * decay > 0.  Writes the right-hand side (N x nrhs, ldb) if B != NULL. */
HODLR_API int hodlr_generate(hodlr_handle h, uint64_t seed, double shift, int orthonormal,
                   double decay, double *B, int64_t ldb, int nrhs);

/* Phases of the per-phase device timing (hodlr_profile). */
enum {
  HODLR_PHASE_LEAF_LU = 0,       /* K1 leaf getrf */
  HODLR_PHASE_LEAF_SOLVE = 1,    /* K2 leaf getrs */
  HODLR_PHASE_REDUCE = 2,        /* K3 A^T X reductions of the sweeps */
  HODLR_PHASE_CAPACITANCE = 3,   /* K4 capacitance LU / solves */
  HODLR_PHASE_UPDATE = 4,        /* K5 low-rank updates of the sweeps */
  HODLR_PHASE_RESID_LEAF = 5,    /* residual: leaf blocks */
  HODLR_PHASE_RESID_REDUCE = 6,  /* residual: V^T x reductions */
  HODLR_PHASE_RESID_UPDATE = 7,  /* residual: U (s . t) updates */
  HODLR_PHASE_MISC = 8,          /* conversions, splits, norms */
  HODLR_NUM_PHASES = 9
};

/* Per-phase device timing: enable = 1 / 0 switches CUDA-event timing of
 * every launch (by phase) on or off (-1 leaves it); if phase_ms /
 * phase_launches are given, the sums since the last read are copied out
 * (nphase entries) and reset. */
HODLR_API int hodlr_profile(hodlr_handle h, int enable, double *phase_ms, int64_t *phase_launches,
                            int nphase);

/* Milliseconds the last hodlr_factor / hodlr_solve spent on the device
 * (CUDA events on the handle's stream). */
HODLR_API int hodlr_last_timings(hodlr_handle h, double *factor_ms, double *solve_ms);

/* ------------------------------------------------------- ragged batches
 * Many independent HODLR systems of different sizes, leaf sizes, ranks and
 * right-hand-side counts, factored and solved together.  No counterpart in
 * the reference, which builds one tree per HMatrix (include/hmatrix.hpp:
 * 10-23) and runs its leaves and nodes as separate Legion tasks
 * (src/lmatrix.cc:449-865); the per-system arithmetic is that of
 * hodlr_factor / hodlr_solve.  Systems sharing (leaf, rank) are stacked into
 * one forest whose levels are processed by single launches over all its
 * trees; the forests run as concurrent branches of one CUDA graph, so after
 * the first call a factorisation or a solve of the whole batch is one graph
 * launch. */
typedef struct hodlr_system {
  int64_t n;       /* leaf * 2^levels */
  int32_t leaf;    /* leaf block size m */
  int32_t levels;  /* tree depth L (0: one dense block) */
  int32_t rank;    /* rank of every off-diagonal block, 1..64 (ignored when levels = 0) */
  int32_t nrhs;    /* right-hand sides solved per call, >= 1 */
} hodlr_system;

typedef struct hodlr_batch_desc {
  const hodlr_system *systems;
  int32_t count;
  int32_t precision;       /* HODLR_PREC_FP64 or HODLR_PREC_MIXED (all systems) */
  int32_t residual;        /* HODLR_RESID_* (mixed only) */
  double refine_tol;       /* per system: max_j ||r_j|| / ||b_j|| */
  int32_t refine_max_iter;
  int32_t flags;           /* reserved, 0 */
  void *stream;            /* cudaStream_t the batch is ordered on, or NULL (own stream) */
} hodlr_batch_desc;

typedef struct hodlr_batch_ctx *hodlr_batch;

HODLR_API int hodlr_batch_create(const hodlr_batch_desc *desc, hodlr_batch *out);
HODLR_API int hodlr_batch_destroy(hodlr_batch b);
/* System i's leaf blocks and level-l factors, with the meaning and layouts
 * of hodlr_set_leaf_blocks / hodlr_set_lowrank (host or device memory).
 * s, when given, is folded into V at set time (V diag(s)). */
HODLR_API int hodlr_batch_set_leaf_blocks(hodlr_batch b, int i, const double *D, int64_t ld,
                                          int64_t leaf_stride);
HODLR_API int hodlr_batch_set_lowrank(hodlr_batch b, int i, int level, const double *U, int64_t ldu,
                                      const double *V, int64_t ldv, const double *s);
/* Seeded random systems (system i seeded with seed + i): leaves
 * G/sqrt(m) + shift I, U and V Gaussian scaled by 1/sqrt(block rows), and,
 * if B is given, Gaussian right-hand sides B[i] (n_i x nrhs_i, ld ldb[i]). */
HODLR_API int hodlr_batch_generate(hodlr_batch b, uint64_t seed, double shift, double *const *B,
                                   const int64_t *ldb);
HODLR_API int hodlr_batch_factor(hodlr_batch b);
/* X_i = A_i^{-1} B_i for every system, in place: B[i] is a device pointer
 * to n_i x nrhs_i column-major values with leading dimension ldb[i].  info
 * (count entries, or NULL) receives each system's status, refinement
 * iterations (of its forest) and, in mixed mode, its relative residual. */
HODLR_API int hodlr_batch_solve(hodlr_batch b, double *const *B, const int64_t *ldb, hodlr_solve_info *info);
/* Forests the batch was split into, and device milliseconds of the last
 * hodlr_batch_factor / hodlr_batch_solve. */
HODLR_API int hodlr_batch_stats(hodlr_batch b, int *nforests, double *factor_ms, double *solve_ms);

/* ------------------------------------------------------------ autotuner
 * Launch shapes of the tunable kernels: the split-K target of the row
 * reductions (CTAs per SM), the row tile of the FP32-FMA low-rank update,
 * the tile and ring depth of the tensor-core update, the warps per
 * capacitance system of the mixed path and the kernel of its leaf
 * application (tensor cores or FP32-FMA tiles).
 * No counterpart in the reference (its BLAS calls have no launch shapes).
 * hodlr_autotune times complete factor + solve sweeps of the handle's own
 * inputs (a seeded scratch right-hand side of nrhs columns) for a coordinate
 * search over the candidates, keeps the fastest and leaves the handle
 * factored with it; choices change only rounding, not the algorithm.  Its
 * result can be cached by the caller and restored with hodlr_set_tuning
 * (which invalidates the factorisation).  hodlr_batch_autotune does the same
 * per forest (systems sharing leaf size and rank); the batch must be
 * factored again afterwards. */
typedef struct hodlr_tuning {
  int32_t red_ctas_per_sm;   /* 2, 4 or 8 */
  int32_t update_tile_rows;  /* 0 (128 where the blocks allow it, else 64) or 64 */
  int32_t cap_warps;         /* mixed path, 2r <= 64: warps per capacitance system, 8, 16 or 32
                                (0 = by level: 32 up to one system per SM, 16 up to two, else 8) */
  int32_t update_tc_shape;   /* tensor-core update: 0 = 128x64 tiles through a 3-stage ring,
                                1 = 128x64 tiles, 2 stages, 2 = 128x32 tiles, 5 stages */
  int32_t leaf_apply;        /* mixed path, leaf 128: the factorisation's application D^-1 U on
                                the tensor cores (0) or on the FP32 FMA pipe (1) */
  double ms;                 /* autotune: factor + solve milliseconds with these shapes */
} hodlr_tuning;

HODLR_API int hodlr_autotune(hodlr_handle h, int nrhs, hodlr_tuning *best);
HODLR_API int hodlr_set_tuning(hodlr_handle h, const hodlr_tuning *t);
HODLR_API int hodlr_get_tuning(hodlr_handle h, hodlr_tuning *t);
HODLR_API int hodlr_batch_autotune(hodlr_batch b, hodlr_tuning *per_forest, int capacity);

/* ------------------------------------------------------ irregular trees
 * One HODLR matrix whose top T levels join 2^T uniform subtrees, each with
 * its own leaf size, depth, rank and precision, and whose top nodes may
 * couple their children with unequal ranks -- the matrices of fastSolver2's
 * SPMD drivers without padding: spmd_driver/solver.cc (one subtree per
 * shard under spmd_level top levels), solver_irregular_part.cc:73-79 (the
 * first `-heavy` shards with ten times the leaf size) and
 * solver_irregular_ranks.cc:99-132 (shard ranks rank0 / rank1, top coupling
 * bases with the sibling's rank).  Top node p (depth l, position q,
 * p = 2^l - 1 + q) with children c0, c1 holds
 *     A[c0,c1] = U_c0 V_c1^T  (rank coupling_rank[2p]),
 *     A[c1,c0] = U_c1 V_c0^T  (rank coupling_rank[2p+1]),
 * and the factorisation solves each node's (r0+r1)-square system as
 * hodlr_node_solve_irregular does.  The subtrees are handles of their own
 * (set their leaf blocks and bases with the hodlr_set_* calls on the handle
 * hodlr_tree_subtree returns); the top levels run in FP64.  Rows are the
 * subtrees' rows in order (hodlr_tree_rows). */
typedef struct hodlr_tree_desc {
  int32_t top_levels;             /* T, 1..7 */
  const hodlr_desc *subtrees;     /* 2^T subtree descriptions, left to right;
                                     nrhs_max and stream are set by the tree */
  const int32_t *coupling_rank;   /* 2 (2^T - 1) ranks, each 1..64 */
  int32_t nrhs_max;               /* largest nrhs of a solve or product */
  int32_t flags;                  /* reserved, 0 */
  void *stream;                   /* cudaStream_t, or NULL (own stream) */
} hodlr_tree_desc;

typedef struct hodlr_tree_ctx *hodlr_tree;

HODLR_API int hodlr_tree_create(const hodlr_tree_desc *desc, hodlr_tree *out);
HODLR_API int hodlr_tree_destroy(hodlr_tree t);
/* Subtree j's handle (owned by the tree; do not destroy it). */
HODLR_API int hodlr_tree_subtree(hodlr_tree t, int j, hodlr_handle *out);
/* Total rows n and, if row_offsets is given, the first row of every subtree
 * (2^T + 1 entries, the last = n). */
HODLR_API int hodlr_tree_rows(hodlr_tree t, int64_t *n, int64_t *row_offsets);
/* Coupling bases of child `child` (0 or 1) of top node (level, pos): U_c
 * (rows of c x its own rank) and V_c (rows of c x the sibling's rank), the
 * child's rows packed from its first row; leading dimensions ldu, ldv.  Host
 * or device memory. */
HODLR_API int hodlr_tree_set_coupling(hodlr_tree t, int level, int pos, int child, const double *U, int64_t ldu,
                                      const double *V, int64_t ldv);
/* Subtree factorisations, U~ = A_sub^{-1} U of every coupling column, and
 * the top nodes' LU factors, deepest level first. */
HODLR_API int hodlr_tree_factor(hodlr_tree t);
/* X = A^{-1} B in place (device, n x nrhs, ldb).  info: the largest
 * refinement count and relative residual over the subtrees' own solves. */
HODLR_API int hodlr_tree_solve(hodlr_tree t, double *B, int64_t ldb, int nrhs, hodlr_solve_info *info);
/* Y = A X in FP64 from the exact representation (device). */
HODLR_API int hodlr_tree_matvec(hodlr_tree t, const double *X, int64_t ldx, double *Y, int64_t ldy, int nrhs);

/* Test hook of the bounded device waits (no counterpart in the reference,
 * whose CPU tasks have no device waits).  While set (cta >= 0), CTA `cta` of
 * every launch of the FP32 row-reduction kernels (the TMA-fed V^T X of the
 * mixed path, on the tensor cores or on the FMA pipe) does not issue the
 * copies of its stage `stage` (counted over the CTA's launch), so its wait on
 * that stage ends only by a clock budget of `budget_cycles` SM cycles
 * (1 .. 1e9; 0 = the default of 1e9): the CTA records HODLR_ERR_TIMEOUT with
 * its index in the handle's status word, waits (bounded) for its copies in
 * flight and returns, and the call reports the error.  cta = -1 switches the
 * hook off.  Affects the current device; no allocation, synchronous. */
HODLR_API int hodlr_debug_wait_fault(int cta, int stage, long long budget_cycles);

/* Kernels launched by this library since load (for launch accounting). */
HODLR_API int64_t hodlr_kernel_launches(void);

HODLR_API const char *hodlr_last_error_string(void);

#ifdef __cplusplus
}
#endif
#endif /* HODLR_GB300_H */
