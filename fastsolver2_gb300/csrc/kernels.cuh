// Launchers of the HODLR kernels (host side).  Every launcher enqueues on
// the given stream and returns the launch error (if any).
#pragma once
#include "common.cuh"

namespace hodlr {

// Record the message returned by hodlr_last_error_string(); returns code.
int set_last_error(int code, const char *msg);

// Launch-shape choices of the tunable kernels, chosen per handle (per forest
// of a batch) by the autotuner.  Launches made by a host thread use the
// choices of the innermost live TuningScope on that thread (defaults
// otherwise).
struct Tuning {
  int red_ctas_per_sm = 4;  // split-K target of the row reductions, CTAs per SM (2, 4 or 8)
  int upd_bm = 0;           // FP32 update tile rows: 0 = 128 when the block allows, else 64
  int cap_warps = 0;        // mixed-path capacitance LU (2r <= 64): warps per node, 8, 16 or 32 (0: by level)
  int upd_tc_shape = 0;     // tcgen05 update: 0 = 128x64 tiles, 3-stage ring; 1 = 128x64, 2 stages; 2 = 128x32, 5 stages
  int leaf_apply = 0;       // mixed factorisation's D^-1 U, leaf 128: 0 = tcgen05 kernel, 1 = FP32-FMA kernel
};
constexpr int kMaxRedCtasPerSm = 8;
constexpr int kNumSMs = 152;
const Tuning &current_tuning();
// CTAs of a persistent launch over `units` work items: one per SM, at most
// one per unit.  The persistent kernels stride over their units by the grid
// size and write per unit, so the grid changes only how the units are shared
// out, never the results.
long long persistent_ctas(long long units);
struct TuningScope {
  const Tuning *prev;
  explicit TuningScope(const Tuning *t);
  ~TuningScope();
};

// ------------------------------------------------------------------ leaves
// K1: LU with partial pivoting of every leaf block.  D: leaf i at
// D + i*d_stride (FP64, column-major, ld d_ld).  LU: packed [nleaf][m][m]
// of type T.  ipiv: [nleaf][m], 1-based.  Zero pivots / non-finite entries
// are reported in *st.
// Dinv (may be NULL): also write the explicit inverses, formed from the
// factors while they are still in shared memory (leaf_getrf_fused_inverse).
bool leaf_getrf_fused_inverse(int m, int elem_bytes);
// FP32 explicit inverses of nleaf leaf blocks of 128 rows (FP64 source in
// the layout of launch_leaf_getrf) by blocked Gauss-Jordan with implicit row
// pivoting; no LU factors.  A zero pivot is reported as HODLR_ERR_SINGULAR_LEAF.
cudaError_t launch_leaf_gj_inverse_f32(const double *D, long long d_ld, long long d_stride, int m, int nleaf,
                                       DevStatus *st, float *Dinv, cudaStream_t s);
template <typename T>
cudaError_t launch_leaf_getrf(const double *D, long long d_ld, long long d_stride, T *LU, int *ipiv,
                              int m, int nleaf, DevStatus *st, T *Dinv, cudaStream_t s);

// The same factorisation for leaves too large for one CTA's shared memory:
// blocked right-looking LU over panels of 32 columns, each panel step one
// launch over the leaves and one over (trailing column tile, leaf).
template <typename T>
cudaError_t launch_leaf_getrf_blocked(const double *D, long long d_ld, long long d_stride, T *LU, int *ipiv, int m,
                                      int nleaf, DevStatus *st, cudaStream_t s);

// Explicit inverses from those factors for leaves whose LU does not fit one
// CTA's shared memory: (32-column tile, leaf) CTAs, blocked triangular solves
// of the interchanged identity.  Shared memory per CTA:
// leaf_inverse_blocked_smem(m, sizeof(T)).
size_t leaf_inverse_blocked_smem(int m, int elem_bytes);
template <typename T>
cudaError_t launch_leaf_inverse_blocked(const T *LU, const int *ipiv, int m, int nleaf, T *Dinv, cudaStream_t s);

// K2: X := D_i^{-1} X (or D_i^{-T} X) on the rows of every leaf i for the
// columns [0, ncols) of X (ld ldx).  skip (device flag, may be NULL): when
// *skip != 0 the kernel returns immediately.
template <typename T>
cudaError_t launch_leaf_getrs(const T *LU, const int *ipiv, int m, int nleaf, T *X, long long ldx,
                              int ncols, bool trans, const int *skip, cudaStream_t s);

// ----------------------------------------------------------- level steps
// K3: Out_b = A_b^T X_b (r x C, FP64 result) for batches b in [0, nbatch),
// A_b / X_b = rows [b*nrows, (b+1)*nrows) of A (N x r, lda) / X (N x C, ldx).
// Split over row chunks with a deterministic second pass.  Out: [nbatch]
// blocks of r x C column-major (ld r); with out32 set, the result goes there
// in FP32 instead.  work: scratch of at least reduce_workspace_doubles(...)
// doubles.
size_t reduce_workspace_doubles(long long nrows, int nbatch, int r, int C, int elem_bytes);
// The row reduction of FP32 operands on the tcgen05 tensor cores (rank <= 32;
// launched when its preconditions hold, else false and nothing launched).
template <typename OutT>
bool reduce_tc_try(const float *V, long long ldv, const float *X, long long ldx, long long nrows, int nbatch, int r,
                   int C, int chunk_rows, int nchunks, OutT *dst, const int *skip, DevStatus *st, cudaStream_t s,
                   cudaError_t &err);

// Test hook of the bounded waits (set by hodlr_debug_wait_fault, off in
// normal use): CTA `cta` of every launch of the FP32 row-reduction kernels
// does not issue the copies of its stage `stage`, so nothing ever completes
// that stage's mbarrier phase and the CTA's wait on it can only end by its
// clock budget, `budget` cycles for that CTA (0 = the default budget; every
// other CTA keeps the default).  Each kernel's file holds its own device copy.
struct WaitFault {
  int cta, stage;
  long long budget;
};
cudaError_t reduce_tc_set_wait_fault(const WaitFault &wf);
template <typename T>
cudaError_t launch_reduce_tn(const T *A, long long lda, const T *X, long long ldx, long long nrows,
                             int nbatch, int r, int C, double *out, double *work, const int *skip,
                             cudaStream_t s, DevStatus *st = nullptr, float *out32 = nullptr);

// K5: C_b += alpha * A_b * diag(scale) * op(B_b) for b in [0, nbatch):
//   A_b = A + b*a_bstride (M x K, lda), C_b = C + b*c_bstride (M x N, ldc),
//   B_b = B + (b >> 1) * b_s1 + ((b & 1) ^ b_flip) * b_s2 (FP64), op(B_b) is
//   K x N: element (q, j) at B_b[q + j*ldb] (b_trans = 0) or B_b[j + q*ldb].
//   scale (optional, FP64) multiplies the inner index q (scale_cols = 0) or
//   the output column j (scale_cols = 1).
struct UpdateArgs {
  const void *A; long long lda; long long a_bstride; int a_trans;  // a_trans: A_b(i,q) at A_b[q + i*lda]
  const double *B; long long ldb; long long b_s1, b_s2; int b_flip; int b_trans;
  const float *B32;  // FP32 kernels: if set, B is read from here (same layout, scale already applied)
  const double *scale; int scale_cols;
  void *C; long long ldc; long long c_bstride;
  int M, N, K, nbatch;
  double alpha;
  const int *skip;
};
template <typename T>
cudaError_t launch_update_nn(const UpdateArgs &a, cudaStream_t s, DevStatus *st = nullptr);

// Explicit inverses of the leaf blocks from their LU factors ([nleaf][m][m]).
template <typename T>
cudaError_t launch_leaf_inverse(const T *LU, const int *ipiv, int m, int nleaf, T *Dinv, cudaStream_t s);
// X_i := op(Dinv_i) X_i on the rows of every leaf (m in {64, 128, 256}).
bool leaf_apply_supported(int m);
template <typename T>
cudaError_t launch_leaf_apply(const T *Dinv, int m, int nleaf, T *X, long long ldx, int ncols, bool trans,
                              const int *skip, cudaStream_t s);
// X := Dinv X for leaf size 128 with the source read from Xs (FP64, leading
// dimension lds) and rounded to FP32 as it is staged (the factorisation's
// U -> Utilde): on the tcgen05 tensor cores where the tensor map can be made,
// else on the FMA pipe; cudaErrorNotSupported for other leaf sizes.
cudaError_t launch_leaf_apply_f64src(const float *Dinv, int m, int nleaf, const double *Xs, long long lds, float *X,
                                     long long ldx, int ncols, DevStatus *st, cudaStream_t s);
// The tcgen05 path of the above (false: preconditions not met, nothing launched).
bool leaf_apply_tc_try(const float *Dinv, int nleaf, const double *U, long long lds, float *Y, long long ldy,
                       int ncols, DevStatus *st, cudaStream_t s, cudaError_t &err);

// Capacitance factorisation of the nodes of one depth: S from the T blocks'
// columns [ucol, ucol + r), FP64 LU (stored in cap_lu / cap_ipiv) and the FP64
// inverse Sinv (plus its double-word split in sinv2 when given).
struct CapFactorArgs {
  const double *Tb; long long tb_stride;
  const float *Tb32;  // if set, the T blocks are read from here (FP32, same layout)
  const double *scale;
  int ucol;
  double *cap_lu; int *cap_ipiv;
  double *sinv; float2 *sinv2;
  float *sinv32;  // mixed path: LU in FP64 only, the inverse in FP32 (from S) written here instead
  int r, nnode, node_base;
  DevStatus *st;
};
cudaError_t launch_cap_factor(const CapFactorArgs &a, cudaStream_t s);

// eta_p = op(Sinv_p) RHS_p (2r x C per node, ld 2r) with RHS_p built from the
// T blocks (forward: [s.T1; s.T0], transposed: [T0; T1]).  Double-word
// arithmetic on the FP32 pipes when sinv2 is given, DFMA otherwise.
struct CapApplyArgs {
  const double *Tb; long long tb_stride;
  const float *Tb32;      // mixed path: FP32 T blocks, applied with the FP32 inverse sinv32
  const float *sinv32;
  const double *scale;
  const double *sinv; const float2 *sinv2;
  double *eta;
  float *eta32;              // if set: FP32 output instead, rows scaled by out_scale[i % r]
  const double *out_scale;   // (for FP32 consumers; may be null)
  int r, C, nnode, node_base;
  bool trans;
  const int *skip;
};
cudaError_t launch_cap_apply(const CapApplyArgs &a, cudaStream_t s);

// --------------------------------------------------------------- helpers
// Y[i, j] = (T) X[i, j] for an n x c column-major tile.
template <typename Tin, typename Tout>
cudaError_t launch_convert(const Tin *X, long long ldx, Tout *Y, long long ldy, long long n, int c,
                           cudaStream_t s);
// Pack leaf blocks (leaf i at D + i*stride, ld) into [nleaf][m][m].
cudaError_t launch_pack_leaves(const double *D, long long ld, long long stride, double *out, int m,
                               int nleaf, cudaStream_t s);
// Inverse of launch_pack_leaves: [nleaf][m][m] (type T) into leaf i at
// out + i*stride (FP64, ld).
template <typename T>
cudaError_t launch_unpack_leaves(const T *in, double *out, long long ld, long long stride, int m, int nleaf,
                                 cudaStream_t s);
// Y = X (FP64 copy of an n x c tile), optionally accumulate: Y += alpha*X.
cudaError_t launch_axpy(const double *X, long long ldx, double *Y, long long ldy, long long n, int c,
                        double alpha, bool accumulate, const int *skip, cudaStream_t s);
// Y = X + (double) D  (FP64 accumulate a lower-precision correction), Y may alias X.
template <typename Td>
cudaError_t launch_add_correction(const double *X, long long ldx, const Td *D, long long ldd,
                                  double *Y, long long ldy, long long n, int c, const int *skip,
                                  cudaStream_t s);
// Column norms ||X_j||_2 (FP64) into out[j]; deterministic.
cudaError_t launch_colnorms(const double *X, long long ldx, long long n, int c, double *out,
                            double *work, const int *skip, cudaStream_t s);
// Per-system column norms of a forest: out[j*nsys + i] = ||rows of system i
// in column j||_2, system i = leaves [seg_leaf[i], seg_leaf[i+1]) of m rows.
// work: nleaf*c doubles.  Deterministic.
cudaError_t launch_seg_colnorms(const double *X, long long ldx, int m, int nleaf, int c, const int *seg_leaf,
                                int nsys, double *out, double *work, const int *skip, cudaStream_t s);
// Fused refinement passes.  Partial sums of squares go to work[j * P + p]
// for P row blocks (P = 64 for one system; P = nleaf, one leaf per block, for
// a forest), and launch_partial_norms turns them into column norms (seg =
// nullptr) or per-system norms (seg = the systems' leaf offsets).
//   rhs_prepare:  B64 = B, X32 = fl32(B)
//   resid_finish: X32 = fl32(hi + lo) of the double-word residual R2
cudaError_t launch_rhs_prepare(const double *B, long long ldb, long long n, int k, int P, double *B64, float *X32,
                               double *work, cudaStream_t s);
cudaError_t launch_resid_finish(const float2 *R2, long long n, int k, int P, float *X32, double *work,
                                const int *skip, cudaStream_t s);
cudaError_t launch_partial_norms(const double *work, int P, int k, const int *seg, int nseg, double *out,
                                 const int *skip, cudaStream_t s);
// X[:, j] *= sc[j] for the n x c tile X (FP64).
cudaError_t launch_scale_cols(double *X, long long ldx, long long n, int c, const double *sc, cudaStream_t s);
// Right-hand sides of the systems of a ragged batch and the stacked n x kmax
// block of their forest: system i owns rows [row_off, row_off + n) and
// columns [0, k) of its own buffer ext (ld).
struct RhsCopy {
  double *ext;
  long long ld, row_off, n;
  int k, pad;
};
// G[row_off + i, j] = ext[i, j] for j < k, 0 for k <= j < kmax (every system in tab).
cudaError_t launch_gather_rhs(const RhsCopy *tab, int count, long long maxn, double *G, long long ldg, int kmax,
                              cudaStream_t s);
// ext[i, j] = G[row_off + i, j] for j < k.
cudaError_t launch_scatter_rhs(const RhsCopy *tab, int count, long long maxn, const double *G, long long ldg,
                               int kmax, cudaStream_t s);
// Refinement control: rel = max_j rnorm[j]/bnorm[j]; st->resid = rel;
// if rel <= tol set st->done = 1.  If advance, count an iteration when not done.
cudaError_t launch_refine_check(const double *rnorm, const double *bnorm, int c, double tol,
                                DevStatus *st, int advance, cudaStream_t s);
// The same check inside a captured graph's refinement loop: unless done, a
// correction is counted while fewer than maxit were applied, and the graph's
// loop condition `cond` is set to whether one follows.
cudaError_t launch_refine_check_cond(const double *rnorm, const double *bnorm, int c, double tol, DevStatus *st,
                                     int maxit, cudaGraphConditionalHandle cond, cudaStream_t s);
// Scan X (n x c) for NaN/Inf; report HODLR_ERR_NONFINITE_INPUT with the row.
cudaError_t launch_check_finite(const double *X, long long ldx, long long n, int c, DevStatus *st,
                                cudaStream_t s);
cudaError_t launch_fill(double *X, long long n, double v, cudaStream_t s);
// D_i[j, j] += d[i*m + j] for the packed leaf blocks [nleaf][m][m].
cudaError_t launch_add_leaf_diag(double *D, const double *d, int m, int nleaf, cudaStream_t s);

// ds[j] = -sum_b sum_q W_b[j, q] * T_{b^1}[j, q] (blocks r x k, ld r), FP64.
cudaError_t launch_scale_grad(const double *W, const double *T, int r, int k, int nbatch, double *ds,
                              cudaStream_t s);

// ------------------------------------------------------------- generator
// Counter-based N(0,1) samples: X[i + j*ld] = scale * g(seed, stream, i + j*n).
cudaError_t launch_gaussian(double *X, long long ld, long long n, int c, unsigned long long seed,
                            unsigned long long stream, double scale, cudaStream_t s);
// Leaf blocks [nleaf][m][m] = G/sqrt(m) + shift*I.
cudaError_t launch_gen_leaves(double *D, int m, int nleaf, unsigned long long seed, double shift,
                              cudaStream_t s);
// Unequal leaf sizes embedded in the uniform tree: rows of leaf i (packed at
// off[i], sz[i] rows) to rows i*mp.. of the padded matrix (zero padding), or
// back (unpad); leaf blocks packed one after another (block i at boff[i],
// sz[i] x sz[i]) into [nleaf][mp][mp] with an identity on the padding.
// off, sz, boff are device arrays.
cudaError_t launch_pad_rows(const long long *off, const int *sz, int nleaf, int mp, int cols, const double *src,
                            long long lds, double *dst, long long ldd, bool unpad, cudaStream_t s);
cudaError_t launch_pad_leaf_blocks(const long long *boff, const int *sz, int nleaf, int mp, const double *src,
                                   double *dst, cudaStream_t s);
// The reference's drand48 generator (POSIX 48-bit LCG): srand48 seeding,
// one step, and the state after t steps (the affine map powered by squaring;
// the maps x -> a^k x + c_k commute, so the order of composition is free).
constexpr unsigned long long kLcgA = 0x5DEECE66Dull, kLcgC = 0xBull, kLcgMask = (1ull << 48) - 1;
__host__ __device__ inline unsigned long long lcg_seed(long long seed) {
  return (((unsigned long long)seed & 0xffffffffull) << 16) | 0x330Eull;
}
__host__ __device__ inline unsigned long long lcg_step(unsigned long long x) {
  return (kLcgA * x + kLcgC) & kLcgMask;
}
__host__ __device__ inline unsigned long long lcg_jump(unsigned long long x, unsigned long long t) {
  unsigned long long a = kLcgA, c = kLcgC, A = 1, C = 0;
  while (t) {
    if (t & 1) {
      A = (a * A) & kLcgMask;
      C = (a * C + c) & kLcgMask;
    }
    c = (a * c + c) & kLcgMask;
    a = (a * a) & kLcgMask;
    t >>= 1;
  }
  return (A * x + C) & kLcgMask;
}
// Partition k (rows [k*rows, (k+1)*rows) of A, cols columns, ld lda) filled
// in row-major order from the drand48 stream seeded by seeds[k] (device
// array), each draw plus offset.
cudaError_t launch_rand_block(const long long *seeds, int npart, long long rows, int cols, double offset,
                              double *A, long long lda, cudaStream_t s);
// Leaf blocks [nleaf][m][m] = U_k V_k^T + diag(D_k) in the reference's BLAS
// order, without fused multiply-adds (U, V: n x r, ld n; Dg: n entries).
cudaError_t launch_seeded_leaves(const double *U, const double *V, const double *Dg, long long n, int m, int r,
                                 int nleaf, double *K, cudaStream_t s);
// Per-block Cholesky of Gram matrices G_b (r x r, ld r) and the inverse of
// the upper factor: Rinv_b (r x r, ld r), G = R^T R.  Reports failure in st.
cudaError_t launch_chol_inv(const double *G, double *Rinv, int r, int nbatch, DevStatus *st,
                            cudaStream_t s);

// ---------------------------------------------------------- residual (FP64 emulated)
// R_b -= D_b X_b (leaf part) and R_c -= U_c (s . V_{c^1}^T X_{c^1}) with
// double-FP32 arithmetic; declared in resid_emul.cu.

}  // namespace hodlr
