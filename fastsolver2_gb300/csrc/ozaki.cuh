// FP64-accurate residual products on the tensor cores by exact slicing
// (the Ozaki scheme; Ozaki, Ogita, Oishi, Rump, "Error-free transformations
// of matrix multiplication by using fast routines of matrix
// multiplication", Numer. Algorithms 59, 2012).
//
// Every FP64 operand is scaled by a power of two per group (a row of U or of
// a leaf block D; 64-row chunks of a column of V, X; a column of the small
// coupling blocks T') and cut into kOzSlices signed 7-bit digits
//     a = 2^E * sum_s d_s 2^(-7(s+1)),   |d_s| <= 127,
// each exactly representable in bf16.  A product of two digits is an integer
// below 2^14, so a bf16 MMA with FP32 accumulation sums up to 1024 of them
// (7 digit pairs x up to 128 terms here) exactly; the pairs of one diagonal
// s + t = d share an accumulator and the seven diagonals are combined in
// double-word (FP32 pair) arithmetic with their exact power-of-two weights.
// The truncation (diagonals d >= 7 and the digits' remainder) is below
// 2^-48 of the row's largest |a| times the column's largest |x| per term --
// the accuracy of the double-word arithmetic it replaces -- at an eighth of
// its FP32-pipe cost (mma.sync bf16 runs at ~8x the FFMA rate here).
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"

namespace hodlr {

constexpr int kOzSlices = 7;   // digits per operand (49 bits)
constexpr int kOzChunk = 64;   // rows per exponent group of the column-scaled operands

// Leaf size and rank the tensor-core residual supports (else the double-word one runs).
inline bool oz_supported(int m, int r) { return m % kOzChunk == 0 && m <= 256 && r >= 8 && r <= 64 && r % 8 == 0; }

// Row-scaled digits.  Row i's entries are A(i, q) = A[(i / rpb) * bstride +
// (i % rpb) * si + q * sq], q < cols; digit s of (i, q) goes to
// out[s * slice_stride + i * ld_out + q]; exps[i] = E_i.
cudaError_t launch_oz_slice_rows(const double *A, long long rpb, long long bstride, long long si, long long sq,
                                 long long rows, int cols, __nv_bfloat16 *out, long long ld_out,
                                 long long slice_stride, int *exps, cudaStream_t s);
// Column-scaled digits per 64-row chunk of an n x c column-major matrix
// (n a multiple of 64): digit s of (i, j) to out[s * slice_stride + j * ld_out
// + i]; exps[(i / 64) * c + j].  The sliced value is X (may be null: zero)
// plus the FP32 add (may be null); xout (may be null) receives it.
cudaError_t launch_oz_slice_cols(const double *X, long long ldx, long long n, int c, __nv_bfloat16 *out,
                                 long long ld_out, long long slice_stride, int *exps, const int *skip,
                                 cudaStream_t s, const float *add = nullptr, double *xout = nullptr);
// Digits of the coupling blocks T'_b = diag(scale) T_{b^1} (r x k blocks of
// T at T + b * r * k, ld r), scaled per column: digit s of (q, j) of block b
// to out[((b * kOzSlices + s) * k + j) * r + q]; exps[b * k + j].
cudaError_t launch_oz_slice_tprime(const double *T, const double *scale, int r, int k, int nb, __nv_bfloat16 *out,
                                   int *exps, const int *skip, cudaStream_t s);

// R2 = split(B) - D X on every leaf (m rows): D digits row-scaled (layout of
// launch_oz_slice_rows with ld_out = m, slice_stride = n m), X digits from
// launch_oz_slice_cols (ld n, slice stride n k).  R2 double-word, ld ldr.
cudaError_t launch_oz_leaf(const __nv_bfloat16 *Dsl, const int *Dexp, int m, int nleaf, const __nv_bfloat16 *Xsl,
                           const int *Xexp, long long n, int k, const double *B, long long ldb, float2 *R2,
                           long long ldr, const int *skip, cudaStream_t s);

// T_b = V_b^T X_b (r x k, FP64) for nb child blocks of `rows` rows from row 0.
// V digits column-scaled (column q of slice s at Vsl + s * vslice + q * n),
// exponents Vexp[(i / 64) * r + q].  Split over row chunks with a
// deterministic second pass.
size_t oz_reduce_workspace_doubles(long long rows, int nb, int r, int k);
cudaError_t launch_oz_reduce(const __nv_bfloat16 *Vsl, long long vslice, const int *Vexp, int r,
                             const __nv_bfloat16 *Xsl, const int *Xexp, long long n, int k, long long rows, int nb,
                             double *out, double *work, const int *skip, cudaStream_t s);

// R2_b -= U_b T'_b for nb child blocks of `rows` rows (U digits row-scaled:
// row i of slice s at Usl + s * uslice + i * r, exps Uexp[i]; T' digits from
// launch_oz_slice_tprime).
cudaError_t launch_oz_update(const __nv_bfloat16 *Usl, long long uslice, const int *Uexp, int r,
                             const __nv_bfloat16 *Tsl, const int *Texp, int k, long long rows, int nb, float2 *R2,
                             long long ldr, const int *skip, cudaStream_t s);

// The T' digits of every level in one launch, from every level's T blocks
// stored one level after another (level l at sum_{l' < l} nb(l') r k); out
// and exps laid out as the tcgen05 residual reads them (below).
constexpr int kOzMaxLevels = 32;
struct TprimeLevels {
  long long wpre[kOzMaxLevels + 1], toff[kOzMaxLevels], ooff[kOzMaxLevels], eoff[kOzMaxLevels];
  const double *scale[kOzMaxLevels];
  int L;
};
cudaError_t launch_oz_slice_tprime_all(const double *T, int r, int k, int L, const int *lev_nb,
                                       const double *const *scale, __nv_bfloat16 *out, int *exps, const int *skip,
                                       cudaStream_t s);

// R2 = split(B) - D X - sum_l U_l T'_l in one pass over 128-row tiles on
// the tcgen05 tensor cores (oz_tc.cu): leaf size 128 or 256, the T' digits
// of every level stored one level after another (level l's block b at line
// offset sum_{l' < l} 7 k nb(l') + 7 k b, exponents at sum_{l' < l} k nb(l')
// + k b); lev_nb / lev_rows: host arrays of the level geometry.
bool oz_tc_supported(int m, int r, int k);
cudaError_t launch_oz_tc_resid(const __nv_bfloat16 *Dsl, const int *Dexp, const __nv_bfloat16 *Xsl, const int *Xexp,
                               const __nv_bfloat16 *Usl, const int *Uexp, const __nv_bfloat16 *Tsl, const int *Texp,
                               long long n, int m, int L, int r, int k, const int *lev_nb, const long long *lev_rows,
                               const double *B, long long ldb, float2 *R2, long long ldr, const int *skip,
                               DevStatus *st, cudaStream_t s);

// T_l = V_l^T X for every level in one pass (oz_tc.cu): level l's blocks at
// T + sum_{l' < l} nb(l') r k (r x k each, ld r); P: partial sums of blocks
// longer than a reduction range, oz_tc_reduce_partials doubles.
size_t oz_tc_reduce_partials(long long n, int L, int r, int k, const int *lev_nb, const long long *lev_rows);
cudaError_t launch_oz_tc_reduce(const __nv_bfloat16 *Vsl, const int *Vexp, const __nv_bfloat16 *Xsl,
                                const int *Xexp, long long n, int L, int r, int k, const int *lev_nb,
                                const long long *lev_rows, double *T, double *P, const int *skip, DevStatus *st,
                                cudaStream_t s);

}  // namespace hodlr
