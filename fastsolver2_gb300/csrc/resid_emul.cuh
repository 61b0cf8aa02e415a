// Double-word (FP32 pair) kernels of the FP64-accurate residual.
#pragma once
#include "common.cuh"

namespace hodlr {

// Y = split(X): each FP64 value into (fl32(a), fl32(a - fl32(a))).
cudaError_t launch_split(const double *X, long long ldx, float2 *Y, long long ldy, long long n, int c,
                         const int *skip, cudaStream_t s);
// X = (double) hi + (double) lo.
cudaError_t launch_merge(const float2 *Y, long long ldy, double *X, long long ldx, long long n, int c,
                         const int *skip, cudaStream_t s);
// T2[e] = split(scale[e % r] * T[e]) over total entries of r-row blocks.
cudaError_t launch_scale_split(const double *T, const double *scale, int r, long long total, float2 *T2,
                               const int *skip, cudaStream_t s);

// Out_b = A_b^T X_b (r x C, FP64), double-word products and sums; same
// batching and split-K scheme as launch_reduce_tn.
size_t dw_reduce_workspace_doubles(long long nrows, int nbatch, int r, int C);
cudaError_t launch_dw_reduce(const float2 *A, long long lda, const float2 *X, long long ldx, long long nrows,
                             int nbatch, int r, int C, double *out, double *work, const int *skip,
                             cudaStream_t s);

struct DwUpdateArgs {
  const float2 *A; long long lda; long long a_bstride; int a_trans;
  const float2 *B; long long ldb; long long b_s1, b_s2; int b_flip;
  float2 *C; long long ldc; long long c_bstride;
  const double *Cinit; long long ldci;   // optional FP64 initial value of C
  int M, N, K, nbatch;
  const int *skip;
};
// C_b = init_b - A_b B_b in double-word arithmetic.
cudaError_t launch_dw_update(const DwUpdateArgs &a, cudaStream_t s);

}  // namespace hodlr
