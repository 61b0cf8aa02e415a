// FP64-accurate residual R = B - op(A) X on the FP32 pipes.
//
// GB300 issues FP64 FMAs at about 1/58 of its FP32 rate (measured: DFMA
// 1.2 TFLOP/s, FFMA 70 TFLOP/s), which makes a native-FP64 residual the most
// expensive step of mixed-precision refinement.  Here every FP64 value a is
// held as a double-word pair (hi, lo) = (fl32(a), fl32(a - hi)) (48-bit
// significand) and products / sums use error-free transformations:
//   hi*hi = p + e exactly (p = hi*hi, e = fma(hi, hi, -p)),
//   S + p = s + t exactly (TwoSum),
// with the small terms (e, t, hi*lo cross products) accumulated in FP32 and
// folded back into the leading word every staged row block.  The result
// matches an FP64 evaluation to about 2^-48 relative to sum|a_i x_i| (checked
// against the native FP64 residual in the tests).  Values must lie inside the
// FP32 exponent range (|a| < 3e38; parts below 1e-31 lose relative accuracy,
// not absolute accuracy).
//
// The residual's structure is the HODLR matvec of the reference's residual
// formula (tests/test.cc:654), generalised to per-level factors:
//   R = split(B) - D X            (per leaf,   m x m times m x k)
//   T_c = V_c^T X_c, R_c -= U_c (s . T_{sibling(c)})   (per level)
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"
#include "resid_emul.cuh"

namespace hodlr {

struct dw {
  float h, l;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &t) {
  s = a + b;
  const float bb = s - a;
  t = (a - (s - bb)) + (b - bb);
}

// acc += a * x with a = (ah, al), x = (xh, xl); acc = (sh, sl).
__device__ __forceinline__ void dw_fma(float ah, float al, float xh, float xl, float &sh, float &sl) {
  const float p = ah * xh;
  const float e = fmaf(ah, xh, -p);
  float s, t;
  two_sum(sh, p, s, t);
  sh = s;
  sl += t + e;
  sl = fmaf(ah, xl, sl);
  sl = fmaf(al, xh, sl);
}

__device__ __forceinline__ void dw_renorm(float &sh, float &sl) {
  float s, t;
  two_sum(sh, sl, s, t);
  sh = s;
  sl = t;
}

__device__ __forceinline__ float2 split_d(double a) {
  const float h = __double2float_rn(a);
  const float l = __double2float_rn(a - (double)h);
  return make_float2(h, l);
}

// c - s in double-word arithmetic
__device__ __forceinline__ float2 dw_sub(float2 c, float sh, float sl) {
  float s, t;
  two_sum(c.x, -sh, s, t);
  t += c.y - sl;
  const float rh = s + t;
  return make_float2(rh, t - (rh - s));
}

// ------------------------------------------------------------------ split
__global__ void split_kernel(const double *X, long long ldx, float2 *Y, long long ldy, long long n, int c,
                             const int *skip) {
  if (skip && *skip) return;
  HODLR_FOR_2D(i, j, n, c) Y[i + j * ldy] = split_d(X[i + j * ldx]);
}

__global__ void merge_kernel(const float2 *Y, long long ldy, double *X, long long ldx, long long n, int c,
                             const int *skip) {
  if (skip && *skip) return;
  HODLR_FOR_2D(i, j, n, c) {
    const float2 v = Y[i + j * ldy];
    X[i + j * ldx] = (double)v.x + (double)v.y;
  }
}

static int grid_for(long long total) {
  return (int)std::max<long long>(1, std::min<long long>(ceil_div(total, 256), 152 * 16));
}

cudaError_t launch_split(const double *X, long long ldx, float2 *Y, long long ldy, long long n, int c,
                         const int *skip, cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH(split_kernel, grid2d(n, c), 256, 0, s, X, ldx, Y, ldy, n, c, skip);
  return cudaGetLastError();
}

cudaError_t launch_merge(const float2 *Y, long long ldy, double *X, long long ldx, long long n, int c,
                         const int *skip, cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH(merge_kernel, grid2d(n, c), 256, 0, s, Y, ldy, X, ldx, n, c, skip);
  return cudaGetLastError();
}

// T2[b] = split(scale . T[b]) for nbatch blocks of r x k (ld r).
__global__ void scale_split_kernel(const double *T, const double *scale, int r, long long total, float2 *T2,
                                   const int *skip) {
  if (skip && *skip) return;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(e % r);
    T2[e] = split_d(scale ? scale[q] * T[e] : T[e]);
  }
}

cudaError_t launch_scale_split(const double *T, const double *scale, int r, long long total, float2 *T2,
                               const int *skip, cudaStream_t s) {
  if (total == 0) return cudaSuccess;
  HODLR_LAUNCH(scale_split_kernel, grid_for(total), 256, 0, s, T, scale, r, total, T2, skip);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ reduce
static constexpr int kCT = 32, kBK = 32;

template <int RT>
__global__ void __launch_bounds__(256)
dw_reduce_kernel(const float2 *__restrict__ A, long long lda, const float2 *__restrict__ X, long long ldx,
                 long long nrows, int r, int C, int chunk_rows, int nchunks, int nct, double *out,
                 const int *skip) {
  if (skip && *skip) return;
  __shared__ float2 sA[kBK][RT + 1];
  __shared__ float2 sX[kBK][kCT + 1];
  long long lin = blockIdx.x;
  const int ct = (int)(lin % nct);
  lin /= nct;
  const int chunk = (int)(lin % nchunks);
  const int b = (int)(lin / nchunks);
  const int c0 = ct * kCT;
  const long long row_begin = (long long)b * nrows + (long long)chunk * chunk_rows;
  const int rows = (int)min((long long)chunk_rows, nrows - (long long)chunk * chunk_rows);
  const int tid = threadIdx.x, tr = tid & 15, tc = tid >> 4;
  float sh[RT / 16][2], sl[RT / 16][2];
#pragma unroll
  for (int a = 0; a < RT / 16; ++a) sh[a][0] = sh[a][1] = sl[a][0] = sl[a][1] = 0.f;
  const float2 *Ab = A + row_begin;
  const float2 *Xb = X + row_begin + (long long)c0 * ldx;
  const float2 z = make_float2(0.f, 0.f);
  // register double buffering: the next row block's loads are in flight
  // while the current one is multiplied
  constexpr int NA = kBK * RT / 256, NX = kBK * kCT / 256;
  float2 ra[NA], rx[NX];
  auto fetch = [&](int i0) {
    const int ib = min(kBK, rows - i0);
#pragma unroll
    for (int u = 0; u < NA; ++u) {
      const int e = tid + 256 * u, i = e % kBK, q = e / kBK;
      ra[u] = (i < ib && q < r) ? Ab[i0 + i + (long long)q * lda] : z;
    }
#pragma unroll
    for (int u = 0; u < NX; ++u) {
      const int e = tid + 256 * u, i = e % kBK, j = e / kBK;
      rx[u] = (i < ib && c0 + j < C) ? Xb[i0 + i + (long long)j * ldx] : z;
    }
  };
  fetch(0);
  for (int i0 = 0; i0 < rows; i0 += kBK) {
#pragma unroll
    for (int u = 0; u < NA; ++u) {
      const int e = tid + 256 * u;
      sA[e % kBK][e / kBK] = ra[u];
    }
#pragma unroll
    for (int u = 0; u < NX; ++u) {
      const int e = tid + 256 * u;
      sX[e % kBK][e / kBK] = rx[u];
    }
    __syncthreads();
    if (i0 + kBK < rows) fetch(i0 + kBK);
#pragma unroll 4
    for (int i = 0; i < kBK; ++i) {
      const float2 x0 = sX[i][tc], x1 = sX[i][tc + 16];
#pragma unroll
      for (int a = 0; a < RT / 16; ++a) {
        const float2 av = sA[i][tr + 16 * a];
        dw_fma(av.x, av.y, x0.x, x0.y, sh[a][0], sl[a][0]);
        dw_fma(av.x, av.y, x1.x, x1.y, sh[a][1], sl[a][1]);
      }
    }
#pragma unroll
    for (int a = 0; a < RT / 16; ++a) {
      dw_renorm(sh[a][0], sl[a][0]);
      dw_renorm(sh[a][1], sl[a][1]);
    }
    __syncthreads();
  }
  double *o = out + ((long long)b * nchunks + chunk) * r * C;
#pragma unroll
  for (int a = 0; a < RT / 16; ++a) {
    const int q = tr + 16 * a;
    if (q >= r) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j = c0 + tc + 16 * h;
      if (j < C) o[q + (long long)j * r] = (double)sh[a][h] + (double)sl[a][h];
    }
  }
}

__global__ void dw_pass2_kernel(const double *__restrict__ partial, int nchunks, long long blk, double *out,
                                const int *skip) {
  if (skip && *skip) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (e >= blk) return;
  const double *p = partial + (long long)b * nchunks * blk + e;
  double s = 0.0;
  for (int c = 0; c < nchunks; ++c) s += p[(long long)c * blk];
  out[(long long)b * blk + e] = s;
}

static void plan(long long nrows, int nbatch, int C, int target, int &nchunks, int &chunk_rows) {
  const int nct = ceil_div(C, kCT);
  const long long base = (long long)nct * nbatch;
  nchunks = 1;
  if (base < target) nchunks = (int)std::min<long long>(ceil_div(target, base), ceil_div(nrows, 256));
  nchunks = std::max(1, nchunks);
  chunk_rows = (int)std::min<long long>(nrows, (long long)ceil_div(ceil_div(nrows, nchunks), kBK) * kBK);
  nchunks = ceil_div(nrows, chunk_rows);
}

size_t dw_reduce_workspace_doubles(long long nrows, int nbatch, int r, int C) {
  int nchunks, chunk_rows;
  plan(nrows, nbatch, C, kMaxRedCtasPerSm * kNumSMs, nchunks, chunk_rows);
  return nchunks > 1 ? (size_t)nbatch * nchunks * r * C : 0;
}

cudaError_t launch_dw_reduce(const float2 *A, long long lda, const float2 *X, long long ldx, long long nrows,
                             int nbatch, int r, int C, double *out, double *work, const int *skip,
                             cudaStream_t s) {
  if (C <= 0 || nbatch <= 0) return cudaSuccess;
  if (r < 1 || r > 64) return cudaErrorInvalidValue;
  int nchunks, chunk_rows;
  plan(nrows, nbatch, C, current_tuning().red_ctas_per_sm * kNumSMs, nchunks, chunk_rows);
  const int nct = ceil_div(C, kCT);
  double *dst = nchunks > 1 ? work : out;
  const long long nblk = (long long)nct * nchunks * nbatch;
#define HODLR_DWR(RT)                                                                                       \
  HODLR_LAUNCH(dw_reduce_kernel<RT>, (unsigned)nblk, 256, 0, s, A, lda, X, ldx, nrows, r, C, chunk_rows, \
               nchunks, nct, dst, skip)
  if (r <= 16) HODLR_DWR(16);
  else if (r <= 32) HODLR_DWR(32);
  else HODLR_DWR(64);
#undef HODLR_DWR
  if (nchunks > 1) {
    const long long blk = (long long)r * C;
    HODLR_LAUNCH(dw_pass2_kernel, dim3(ceil_div(blk, 256), nbatch), 256, 0, s, work, nchunks, blk, out, skip);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------ update
static constexpr int kBM = 64, kBN = 32, kUK = 32;

// C_b = init_b - A_b op(B_b): A_b = A + b*a_bstride (M x K, lda, or its
// transpose when a_trans), B_b = B + (b>>1)*b_s1 + ((b&1)^b_flip)*b_s2
// (K x N, ldb), init_b = split(Cinit_b) (FP64, ldci) when Cinit is given,
// else C_b itself.  All pairs are double-words.
__global__ void __launch_bounds__(256) dw_update_kernel(DwUpdateArgs a, int nrt, int nct) {
  if (a.skip && *a.skip) return;
  __shared__ float2 sA[kUK][kBM + 1];
  __shared__ float2 sB[kUK][kBN + 1];
  long long lin = blockIdx.x;
  const int rt = (int)(lin % nrt);
  lin /= nrt;
  const int ct = (int)(lin % nct);
  const int b = (int)(lin / nct);
  const int i0 = rt * kBM, j0 = ct * kBN;
  const float2 *A = a.A + (long long)b * a.a_bstride;
  const float2 *B = a.B + (long long)(b >> 1) * a.b_s1 + (long long)((b & 1) ^ a.b_flip) * a.b_s2;
  float2 *C = a.C + (long long)b * a.c_bstride;
  const int tid = threadIdx.x, ti = tid & 31, tj = tid >> 5;
  float sh[2][4], sl[2][4];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) sh[u][v] = sl[u][v] = 0.f;
  const float2 z = make_float2(0.f, 0.f);
  for (int q0 = 0; q0 < a.K; q0 += kUK) {
    for (int e = tid; e < kBM * kUK; e += 256) {
      const int i = e % kBM, q = e / kBM;
      sA[q][i] = (i0 + i < a.M && q0 + q < a.K)
                     ? (a.a_trans ? A[(q0 + q) + (long long)(i0 + i) * a.lda] : A[i0 + i + (long long)(q0 + q) * a.lda])
                     : z;
    }
    for (int e = tid; e < kUK * kBN; e += 256) {
      const int q = e % kUK, j = e / kUK;
      sB[q][j] = (q0 + q < a.K && j0 + j < a.N) ? B[(q0 + q) + (long long)(j0 + j) * a.ldb] : z;
    }
    __syncthreads();
#pragma unroll 4
    for (int q = 0; q < kUK; ++q) {
      const float2 a0 = sA[q][ti], a1 = sA[q][ti + 32];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float2 bv = sB[q][tj + 8 * v];
        dw_fma(a0.x, a0.y, bv.x, bv.y, sh[0][v], sl[0][v]);
        dw_fma(a1.x, a1.y, bv.x, bv.y, sh[1][v], sl[1][v]);
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) dw_renorm(sh[u][v], sl[u][v]);
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int i = i0 + ti + 32 * u;
    if (i >= a.M) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = j0 + tj + 8 * v;
      if (j >= a.N) continue;
      float2 *c = C + i + (long long)j * a.ldc;
      const float2 init =
          a.Cinit ? split_d(a.Cinit[(long long)b * a.c_bstride + i + (long long)j * a.ldci]) : *c;
      *c = dw_sub(init, sh[u][v], sl[u][v]);
    }
  }
}

cudaError_t launch_dw_update(const DwUpdateArgs &a, cudaStream_t s) {
  if (a.M <= 0 || a.N <= 0 || a.nbatch <= 0) return cudaSuccess;
  const int nrt = ceil_div(a.M, kBM), nct = ceil_div(a.N, kBN);
  const long long nblk = (long long)nrt * nct * a.nbatch;
  HODLR_LAUNCH(dw_update_kernel, (unsigned)nblk, 256, 0, s, a, nrt, nct);
  return cudaGetLastError();
}

}  // namespace hodlr
