// K3 / K4 / K5: the per-level steps of the HODLR sweep.
//
// fastSolver2 runs these per node on the CPU: V^T [u|d] products
// (src/tasks/leaf_solve.cc:132-135, GemmRedTask src/tasks/gemm_reduce.cc:33-83
// with the Legion Add reduction src/tasks/reduce_add.cc:7-49), the 2r x 2r
// capacitance solve (leaf_solve.cc:118-141, NodeSolveTask
// src/tasks/node_solve.cc:37-82) and d -= u eta (leaf_solve.cc:143-153,
// GemmBroTask src/tasks/gemm_broadcast.cc:33-83).  Here each step covers
// every node of a tree depth in one launch:
//   K3 reduce_tn   -- batched tall-skinny A^T X, split over row chunks with a
//                     deterministic second pass (no atomics: bitwise
//                     reproducible, which doubles as a race check),
//   K4 capacitance -- one CTA per node: build S, LU with partial pivoting and
//                     the solve, all FP64 in shared memory,
//   K5 update_nn   -- batched C += alpha A B with the child/sibling indexing
//                     of the tree folded into the batch addressing.
#include <algorithm>

#include "dense_ops.cuh"
#include "kernels.cuh"

namespace hodlr {

// ------------------------------------------------------------------ K3
static constexpr int kRedCT = 32;   // output columns per CTA
static constexpr int kRedBK = 32;   // rows staged per step
static constexpr int kRedTargetCTAs = 4 * 152;

template <typename T, int RT>
__global__ void __launch_bounds__(256)
reduce_tn_kernel(const T *__restrict__ A, long long lda, const T *__restrict__ X, long long ldx,
                 long long nrows, int r, int C, int chunk_rows, int nchunks, int nct, double *out,
                 const int *skip) {
  if (skip && *skip) return;
  __shared__ T sA[kRedBK][RT + 1];
  __shared__ T sX[kRedBK][kRedCT + 1];
  long long lin = blockIdx.x;
  const int ct = (int)(lin % nct);
  lin /= nct;
  const int chunk = (int)(lin % nchunks);
  const int b = (int)(lin / nchunks);
  const int c0 = ct * kRedCT;
  const long long row_begin = (long long)b * nrows + (long long)chunk * chunk_rows;
  const int rows = (int)min((long long)chunk_rows, nrows - (long long)chunk * chunk_rows);
  const int tid = threadIdx.x, tr = tid & 15, tc = tid >> 4;
  T acc[RT / 16][2];
#pragma unroll
  for (int a = 0; a < RT / 16; ++a) acc[a][0] = acc[a][1] = T(0);
  const T *Ab = A + row_begin;
  const T *Xb = X + row_begin + (long long)c0 * ldx;
  for (int i0 = 0; i0 < rows; i0 += kRedBK) {
    const int ib = min(kRedBK, rows - i0);
    for (int e = tid; e < kRedBK * RT; e += 256) {
      const int i = e % kRedBK, q = e / kRedBK;
      sA[i][q] = (i < ib && q < r) ? Ab[i0 + i + (long long)q * lda] : T(0);
    }
    for (int e = tid; e < kRedBK * kRedCT; e += 256) {
      const int i = e % kRedBK, j = e / kRedBK;
      sX[i][j] = (i < ib && c0 + j < C) ? Xb[i0 + i + (long long)j * ldx] : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int i = 0; i < kRedBK; ++i) {
      const T x0 = sX[i][tc], x1 = sX[i][tc + 16];
#pragma unroll
      for (int a = 0; a < RT / 16; ++a) {
        const T av = sA[i][tr + 16 * a];
        acc[a][0] += av * x0;
        acc[a][1] += av * x1;
      }
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
      if (j < C) o[q + (long long)j * r] = (double)acc[a][h];
    }
  }
}

__global__ void reduce_pass2_kernel(const double *__restrict__ partial, int nchunks, long long blk,
                                    double *out, const int *skip) {
  if (skip && *skip) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (e >= blk) return;
  const double *p = partial + (long long)b * nchunks * blk + e;
  double s = 0.0;
  for (int c = 0; c < nchunks; ++c) s += p[(long long)c * blk];
  out[(long long)b * blk + e] = s;
}

static void reduce_plan(long long nrows, int nbatch, int C, int &nchunks, int &chunk_rows) {
  const int nct = ceil_div(C, kRedCT);
  long long base = (long long)nct * nbatch;
  nchunks = 1;
  if (base < kRedTargetCTAs) nchunks = (int)std::min<long long>(ceil_div(kRedTargetCTAs, base), ceil_div(nrows, 256));
  nchunks = std::max(1, nchunks);
  chunk_rows = (int)std::min<long long>(nrows, (long long)ceil_div(ceil_div(nrows, nchunks), kRedBK) * kRedBK);
  nchunks = ceil_div(nrows, chunk_rows);
}

size_t reduce_workspace_doubles(long long nrows, int nbatch, int r, int C, int) {
  int nchunks, chunk_rows;
  reduce_plan(nrows, nbatch, C, nchunks, chunk_rows);
  return nchunks > 1 ? (size_t)nbatch * nchunks * r * C : 0;
}

template <typename T>
cudaError_t launch_reduce_tn(const T *A, long long lda, const T *X, long long ldx, long long nrows,
                             int nbatch, int r, int C, double *out, double *work, const int *skip,
                             cudaStream_t s) {
  if (C <= 0 || nbatch <= 0) return cudaSuccess;
  if (r < 1 || r > 64) return cudaErrorInvalidValue;
  int nchunks, chunk_rows;
  reduce_plan(nrows, nbatch, C, nchunks, chunk_rows);
  const int nct = ceil_div(C, kRedCT);
  double *dst = nchunks > 1 ? work : out;
  const long long nblk = (long long)nct * nchunks * nbatch;
#define HODLR_RED_CASE(RT)                                                                        \
  HODLR_LAUNCH((reduce_tn_kernel<T, RT>), (unsigned)nblk, 256, 0, s, A, lda, X, ldx, nrows, r, C, \
               chunk_rows, nchunks, nct, dst, skip)
  if (r <= 16) HODLR_RED_CASE(16);
  else if (r <= 32) HODLR_RED_CASE(32);
  else HODLR_RED_CASE(64);
#undef HODLR_RED_CASE
  if (nchunks > 1) {
    const long long blk = (long long)r * C;
    dim3 grid(ceil_div(blk, 256), nbatch);
    HODLR_LAUNCH(reduce_pass2_kernel, grid, 256, 0, s, work, nchunks, blk, out, skip);
  }
  return cudaGetLastError();
}

template cudaError_t launch_reduce_tn<double>(const double *, long long, const double *, long long, long long,
                                              int, int, int, double *, double *, const int *, cudaStream_t);
template cudaError_t launch_reduce_tn<float>(const float *, long long, const float *, long long, long long, int,
                                             int, int, double *, double *, const int *, cudaStream_t);

// ------------------------------------------------------------------ K5
static constexpr int kUpdBM = 64, kUpdBN = 32, kUpdBK = 32;

template <typename T>
__global__ void __launch_bounds__(256) update_nn_kernel(UpdateArgs a, int nrt, int nct) {
  if (a.skip && *a.skip) return;
  __shared__ T sA[kUpdBK][kUpdBM + 1];
  __shared__ T sB[kUpdBK][kUpdBN + 1];
  long long lin = blockIdx.x;
  const int rt = (int)(lin % nrt);
  lin /= nrt;
  const int ct = (int)(lin % nct);
  const int b = (int)(lin / nct);
  const int i0 = rt * kUpdBM, j0 = ct * kUpdBN;
  const T *A = reinterpret_cast<const T *>(a.A) + (long long)b * a.a_bstride;
  const double *B = a.B + (long long)(b >> 1) * a.b_s1 + (long long)((b & 1) ^ a.b_flip) * a.b_s2;
  T *C = reinterpret_cast<T *>(a.C) + (long long)b * a.c_bstride;
  const int tid = threadIdx.x, ti = tid & 31, tj = tid >> 5;
  T acc[2][4];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
  for (int q0 = 0; q0 < a.K; q0 += kUpdBK) {
    for (int e = tid; e < kUpdBM * kUpdBK; e += 256) {
      const int i = e % kUpdBM, q = e / kUpdBM;
      sA[q][i] = (i0 + i < a.M && q0 + q < a.K)
                     ? (a.a_trans ? A[(q0 + q) + (long long)(i0 + i) * a.lda] : A[i0 + i + (long long)(q0 + q) * a.lda])
                     : T(0);
    }
    for (int e = tid; e < kUpdBK * kUpdBN; e += 256) {
      const int q = e % kUpdBK, j = e / kUpdBK;
      double v = 0.0;
      if (q0 + q < a.K && j0 + j < a.N) {
        v = a.b_trans ? B[(j0 + j) + (long long)(q0 + q) * a.ldb] : B[(q0 + q) + (long long)(j0 + j) * a.ldb];
        if (a.scale) v *= a.scale_cols ? a.scale[j0 + j] : a.scale[q0 + q];
      }
      sB[q][j] = (T)v;
    }
    __syncthreads();
#pragma unroll 8
    for (int q = 0; q < kUpdBK; ++q) {
      const T a0 = sA[q][ti], a1 = sA[q][ti + 32];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const T bv = sB[q][tj + 8 * v];
        acc[0][v] += a0 * bv;
        acc[1][v] += a1 * bv;
      }
    }
    __syncthreads();
  }
  const T alpha = (T)a.alpha;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int i = i0 + ti + 32 * u;
    if (i >= a.M) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = j0 + tj + 8 * v;
      if (j < a.N) {
        T *c = C + i + (long long)j * a.ldc;
        *c = *c + alpha * acc[u][v];
      }
    }
  }
}

template <typename T>
cudaError_t launch_update_nn(const UpdateArgs &a, cudaStream_t s) {
  if (a.M <= 0 || a.N <= 0 || a.nbatch <= 0) return cudaSuccess;
  const int nrt = ceil_div(a.M, kUpdBM), nct = ceil_div(a.N, kUpdBN);
  const long long nblk = (long long)nrt * nct * a.nbatch;
  HODLR_LAUNCH(update_nn_kernel<T>, (unsigned)nblk, 256, 0, s, a, nrt, nct);
  return cudaGetLastError();
}
template cudaError_t launch_update_nn<double>(const UpdateArgs &, cudaStream_t);
template cudaError_t launch_update_nn<float>(const UpdateArgs &, cudaStream_t);

// ------------------------------------------------------------------ K4
static constexpr int kCapCT = 32;

__global__ void __launch_bounds__(256) capacitance_kernel(CapArgs a) {
  if (a.skip && *a.skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_info;
  const int p = blockIdx.x;
  const int node = a.node_base + p;
  const int r = a.r, n2 = 2 * r;
  double *S = reinterpret_cast<double *>(smem_raw);
  double *R = S + n2 * n2;
  int *piv = reinterpret_cast<int *>(R + n2 * kCapCT);
  const double *T0 = a.Tb + (long long)(2 * p) * a.tb_stride;
  const double *T1 = a.Tb + (long long)(2 * p + 1) * a.tb_stride;
  auto sc = [&](int i) -> double { return a.scale ? a.scale[i] : 1.0; };
  if (a.factor) {
    for (int e = threadIdx.x; e < n2 * n2; e += blockDim.x) {
      const int i = e % n2, j = e / n2;
      double v = (i == j) ? 1.0 : 0.0;
      if (i >= r && j < r) v = sc(i - r) * T0[(i - r) + (long long)(a.C + j) * r];
      if (i < r && j >= r) v = sc(i) * T1[i + (long long)(a.C + j - r) * r];
      S[e] = v;
    }
    __syncthreads();
    block_getrf<double>(S, n2, n2, piv, &s_info);
    if (s_info && threadIdx.x == 0) report_error(a.st, HODLR_ERR_SINGULAR_CAPACITANCE, node);
    double *gS = a.cap_lu + (long long)node * n2 * n2;
    for (int e = threadIdx.x; e < n2 * n2; e += blockDim.x) gS[e] = S[e];
    for (int e = threadIdx.x; e < n2; e += blockDim.x) a.cap_ipiv[(long long)node * n2 + e] = piv[e];
  } else {
    const double *gS = a.cap_lu + (long long)node * n2 * n2;
    for (int e = threadIdx.x; e < n2 * n2; e += blockDim.x) S[e] = gS[e];
    for (int e = threadIdx.x; e < n2; e += blockDim.x) piv[e] = a.cap_ipiv[(long long)node * n2 + e];
  }
  __syncthreads();
  double *eta = a.eta + (long long)p * n2 * a.C;
  for (int c0 = 0; c0 < a.C; c0 += kCapCT) {
    const int nc = min(kCapCT, a.C - c0);
    for (int e = threadIdx.x; e < n2 * nc; e += blockDim.x) {
      const int i = e % n2, j = e / n2;
      double v;
      if (!a.trans)
        v = (i < r) ? sc(i) * T1[i + (long long)(c0 + j) * r] : sc(i - r) * T0[(i - r) + (long long)(c0 + j) * r];
      else
        v = (i < r) ? T0[i + (long long)(c0 + j) * r] : T1[(i - r) + (long long)(c0 + j) * r];
      R[i + j * n2] = v;
    }
    __syncthreads();
    if (!a.trans)
      block_getrs<double, false>(S, n2, piv, n2, R, n2, nc);
    else
      block_getrs<double, true>(S, n2, piv, n2, R, n2, nc);
    for (int e = threadIdx.x; e < n2 * nc; e += blockDim.x) {
      const int i = e % n2, j = e / n2;
      eta[i + (long long)(c0 + j) * n2] = R[i + j * n2];
    }
    __syncthreads();
  }
}

cudaError_t launch_capacitance(const CapArgs &a, cudaStream_t s) {
  if (a.nnode <= 0) return cudaSuccess;
  if (a.r < 1 || a.r > 64) return cudaErrorInvalidValue;
  const int n2 = 2 * a.r;
  const size_t bytes = (size_t)n2 * n2 * 8 + (size_t)n2 * kCapCT * 8 + (size_t)n2 * 4 + 16;
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(capacitance_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bytes);
    if (e != cudaSuccess) return e;
  }
  HODLR_LAUNCH(capacitance_kernel, a.nnode, 256, bytes, s, a);
  return cudaGetLastError();
}

// --------------------------------------------------------------- helpers
template <typename Tin, typename Tout>
__global__ void convert_kernel(const Tin *X, long long ldx, Tout *Y, long long ldy, long long n, int c) {
  HODLR_FOR_2D(i, j, n, c) Y[i + j * ldy] = (Tout)X[i + j * ldx];
}

static int grid_for(long long total) {
  return (int)std::max<long long>(1, std::min<long long>(ceil_div(total, 256), 152 * 16));
}

template <typename Tin, typename Tout>
cudaError_t launch_convert(const Tin *X, long long ldx, Tout *Y, long long ldy, long long n, int c,
                           cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH((convert_kernel<Tin, Tout>), grid2d(n, c), 256, 0, s, X, ldx, Y, ldy, n, c);
  return cudaGetLastError();
}
template cudaError_t launch_convert<double, float>(const double *, long long, float *, long long, long long,
                                                   int, cudaStream_t);
template cudaError_t launch_convert<float, double>(const float *, long long, double *, long long, long long,
                                                   int, cudaStream_t);
template cudaError_t launch_convert<double, double>(const double *, long long, double *, long long,
                                                    long long, int, cudaStream_t);

__global__ void pack_leaves_kernel(const double *D, long long ld, long long stride, double *out, int m,
                                   long long total) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long mm = (long long)m * m;
    const long long leaf = e / mm, w = e % mm;
    const int i = (int)(w % m), j = (int)(w / m);
    out[e] = D[leaf * stride + i + (long long)j * ld];
  }
}

cudaError_t launch_pack_leaves(const double *D, long long ld, long long stride, double *out, int m,
                               int nleaf, cudaStream_t s) {
  const long long total = (long long)nleaf * m * m;
  HODLR_LAUNCH(pack_leaves_kernel, grid_for(total), 256, 0, s, D, ld, stride, out, m, total);
  return cudaGetLastError();
}

template <typename T>
__global__ void unpack_leaves_kernel(const T *in, double *out, long long ld, long long stride, int m,
                                     long long total) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long mm = (long long)m * m;
    const long long leaf = e / mm, w = e % mm;
    const int i = (int)(w % m), j = (int)(w / m);
    out[leaf * stride + i + (long long)j * ld] = (double)in[e];
  }
}

template <typename T>
cudaError_t launch_unpack_leaves(const T *in, double *out, long long ld, long long stride, int m, int nleaf,
                                 cudaStream_t s) {
  const long long total = (long long)nleaf * m * m;
  HODLR_LAUNCH(unpack_leaves_kernel<T>, grid_for(total), 256, 0, s, in, out, ld, stride, m, total);
  return cudaGetLastError();
}
template cudaError_t launch_unpack_leaves<double>(const double *, double *, long long, long long, int, int,
                                                  cudaStream_t);
template cudaError_t launch_unpack_leaves<float>(const float *, double *, long long, long long, int, int,
                                                 cudaStream_t);

__global__ void axpy_kernel(const double *X, long long ldx, double *Y, long long ldy, long long n, int c,
                            double alpha, int accumulate, const int *skip) {
  if (skip && *skip) return;
  HODLR_FOR_2D(i, j, n, c) {
    const double v = X[i + j * ldx];
    double *y = Y + i + j * ldy;
    *y = accumulate ? *y + alpha * v : alpha * v;
  }
}

cudaError_t launch_axpy(const double *X, long long ldx, double *Y, long long ldy, long long n, int c,
                        double alpha, bool accumulate, const int *skip, cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH(axpy_kernel, grid2d(n, c), 256, 0, s, X, ldx, Y, ldy, n, c, alpha, (int)accumulate, skip);
  return cudaGetLastError();
}

template <typename Td>
__global__ void add_corr_kernel(const double *X, long long ldx, const Td *D, long long ldd, double *Y,
                                long long ldy, long long n, int c, const int *skip) {
  if (skip && *skip) return;
  HODLR_FOR_2D(i, j, n, c) Y[i + j * ldy] = X[i + j * ldx] + (double)D[i + j * ldd];
}

template <typename Td>
cudaError_t launch_add_correction(const double *X, long long ldx, const Td *D, long long ldd, double *Y,
                                  long long ldy, long long n, int c, const int *skip, cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH(add_corr_kernel<Td>, grid2d(n, c), 256, 0, s, X, ldx, D, ldd, Y, ldy, n, c, skip);
  return cudaGetLastError();
}
template cudaError_t launch_add_correction<float>(const double *, long long, const float *, long long, double *,
                                                  long long, long long, int, const int *, cudaStream_t);
template cudaError_t launch_add_correction<double>(const double *, long long, const double *, long long,
                                                   double *, long long, long long, int, const int *,
                                                   cudaStream_t);

// Column sums of squares in two deterministic passes: per (column, slice)
// partial sums, then a fixed-order sum per column.
static constexpr int kNormSlices = 64;

__global__ void colnorm_partial_kernel(const double *X, long long ldx, long long n, double *work,
                                       const int *skip) {
  if (skip && *skip) return;
  const int j = blockIdx.y, sl = blockIdx.x;
  const long long per = (n + kNormSlices - 1) / kNormSlices;
  const long long lo = sl * per, hi = min(n, lo + per);
  double acc = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double v = X[i + (long long)j * ldx];
    acc += v * v;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) work[(long long)j * kNormSlices + sl] = red[0];
}

__global__ void colnorm_final_kernel(const double *work, int c, double *out, const int *skip) {
  if (skip && *skip) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= c) return;
  double s = 0.0;
  for (int k = 0; k < kNormSlices; ++k) s += work[(long long)j * kNormSlices + k];
  out[j] = sqrt(s);
}

cudaError_t launch_colnorms(const double *X, long long ldx, long long n, int c, double *out, double *work,
                            const int *skip, cudaStream_t s) {
  if (c <= 0) return cudaSuccess;
  HODLR_LAUNCH(colnorm_partial_kernel, dim3(kNormSlices, c), 256, 0, s, X, ldx, n, work, skip);
  HODLR_LAUNCH(colnorm_final_kernel, ceil_div(c, 64), 64, 0, s, work, c, out, skip);
  return cudaGetLastError();
}

__global__ void refine_check_kernel(const double *rnorm, const double *bnorm, int c, double tol,
                                    DevStatus *st, int advance) {
  if (threadIdx.x != 0) return;
  if (st->done) return;
  double rel = 0.0;
  for (int j = 0; j < c; ++j) {
    const double b = bnorm[j] > 0.0 ? bnorm[j] : 1.0;
    const double q = rnorm[j] / b;
    rel = (q > rel || q != q) ? q : rel;
  }
  st->resid = rel;
  if (rel <= tol) st->done = 1;
  if (advance && !st->done) st->iters += 1;
}

cudaError_t launch_refine_check(const double *rnorm, const double *bnorm, int c, double tol, DevStatus *st,
                                int advance, cudaStream_t s) {
  HODLR_LAUNCH(refine_check_kernel, 1, 32, 0, s, rnorm, bnorm, c, tol, st, advance);
  return cudaGetLastError();
}

__global__ void check_finite_kernel(const double *X, long long ldx, long long n, int c, DevStatus *st) {
  HODLR_FOR_2D(i, j, n, c) {
    if (!isfinite(X[i + j * ldx])) report_error(st, HODLR_ERR_NONFINITE_INPUT, i);
  }
}

cudaError_t launch_check_finite(const double *X, long long ldx, long long n, int c, DevStatus *st,
                                cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH(check_finite_kernel, grid2d(n, c), 256, 0, s, X, ldx, n, c, st);
  return cudaGetLastError();
}

__global__ void fill_kernel(double *X, long long n, double v) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    X[e] = v;
}

cudaError_t launch_fill(double *X, long long n, double v, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  HODLR_LAUNCH(fill_kernel, grid_for(n), 256, 0, s, X, n, v);
  return cudaGetLastError();
}

__global__ void scale_grad_kernel(const double *W, const double *T, int r, int k, int nbatch, double *ds) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= r) return;
  double acc = 0.0;
  for (int b = 0; b < nbatch; ++b) {
    const double *w = W + (long long)b * r * k;
    const double *t = T + (long long)(b ^ 1) * r * k;
    for (int q = 0; q < k; ++q) acc += w[j + (long long)q * r] * t[j + (long long)q * r];
  }
  ds[j] = -acc;
}

cudaError_t launch_scale_grad(const double *W, const double *T, int r, int k, int nbatch, double *ds,
                              cudaStream_t s) {
  HODLR_LAUNCH(scale_grad_kernel, ceil_div(r, 64), 64, 0, s, W, T, r, k, nbatch, ds);
  return cudaGetLastError();
}

}  // namespace hodlr
