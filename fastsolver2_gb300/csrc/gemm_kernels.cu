// K3 / K5: the batched tall-skinny GEMMs of the sweep.
//
//   K3 reduce_tn  Out_b = A_b^T X_b   (r x C per child; A_b, X_b = the child's
//                 rows of V^(l) or Utilde^(l) and of the right-hand sides) --
//                 the V^T [u|d] products of hsolve (src/tasks/leaf_solve.cc:
//                 132-135) and GemmRedTask (src/tasks/gemm_reduce.cc:33-83).
//   K5 update_nn  C_b += alpha A_b diag(s) op(B_b) -- d -= u eta of hsolve
//                 (leaf_solve.cc:143-153) and GemmBroTask
//                 (src/tasks/gemm_broadcast.cc:33-83); the tree's
//                 child/sibling/node indexing is folded into the batch
//                 addressing of B.
//
// K3 splits the long row dimension three ways: across CTAs (row chunks,
// summed by a deterministic second pass -- no atomics, so results are bitwise
// reproducible run to run), across the four 64-thread groups of a CTA (summed
// in shared memory in a fixed order), and along each thread's rows.  Each
// thread keeps an (RT/8) x 8 register tile; shared-memory rows are padded by
// one element so the column-wise staging stores are bank-conflict free.
#include <algorithm>

#include "kernels.cuh"

namespace hodlr {

// ------------------------------------------------------------------ K3
// output columns per CTA: 64, or 8 for narrow right-hand sides (C <= 8)
static inline int red_bn(int C) { return C <= 8 ? 8 : 64; }
static constexpr int kRedBK = 32;   // rows staged per step
static constexpr int kRedTargetCTAs = 4 * 152;

template <typename T, int RT, int BN>
__global__ void __launch_bounds__(256)
reduce_tn_kernel(const T *__restrict__ A, long long lda, const T *__restrict__ X, long long ldx,
                 long long nrows, int r, int C, int chunk_rows, int nchunks, int nct, double *out,
                 const int *skip) {
  if (skip && *skip) return;
  constexpr int RPT = RT / 8;           // ranks per thread (rows of the output)
  constexpr int CPT = BN / 8;           // columns per thread
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sA = reinterpret_cast<T *>(smem_raw);          // [kRedBK][RT]
  T *sX = sA + kRedBK * (RT + 1);                   // [kRedBK][BN + 1]
  T *sRed = sX + kRedBK * (BN + 1);                 // [4][RT][BN + 1]
  long long lin = blockIdx.x;
  const int ct = (int)(lin % nct);
  lin /= nct;
  const int chunk = (int)(lin % nchunks);
  const int b = (int)(lin / nchunks);
  const int c0 = ct * BN;
  const long long row_begin = (long long)b * nrows + (long long)chunk * chunk_rows;
  const int rows = (int)min((long long)chunk_rows, nrows - (long long)chunk * chunk_rows);
  const int tid = threadIdx.x, g = tid >> 6, t = tid & 63, tr = t & 7, tc = t >> 3;
  T acc[RPT][CPT];
#pragma unroll
  for (int a = 0; a < RPT; ++a)
#pragma unroll
    for (int c = 0; c < CPT; ++c) acc[a][c] = T(0);
  const T *Ab = A + row_begin;
  const T *Xb = X + row_begin + (long long)c0 * ldx;
  for (int i0 = 0; i0 < rows; i0 += kRedBK) {
    const int ib = min(kRedBK, rows - i0);
    for (int e = tid; e < kRedBK * RT; e += 256) {
      const int i = e % kRedBK, q = e / kRedBK;
      sA[i * (RT + 1) + q] = (i < ib && q < r) ? Ab[i0 + i + (long long)q * lda] : T(0);
    }
    for (int e = tid; e < kRedBK * BN; e += 256) {
      const int i = e % kRedBK, j = e / kRedBK;
      sX[i * (BN + 1) + j] = (i < ib && c0 + j < C) ? Xb[i0 + i + (long long)j * ldx] : T(0);
    }
    __syncthreads();
#pragma unroll 2
    for (int ii = 0; ii < kRedBK / 4; ++ii) {
      const int i = ii * 4 + g;
      T av[RPT], xv[CPT];
#pragma unroll
      for (int a = 0; a < RPT; ++a) av[a] = sA[i * (RT + 1) + tr * RPT + a];
#pragma unroll
      for (int c = 0; c < CPT; ++c) xv[c] = sX[i * (BN + 1) + tc * CPT + c];
#pragma unroll
      for (int a = 0; a < RPT; ++a)
#pragma unroll
        for (int c = 0; c < CPT; ++c) acc[a][c] += av[a] * xv[c];
    }
    __syncthreads();
  }
  // fixed-order sum of the four row groups
#pragma unroll
  for (int a = 0; a < RPT; ++a)
#pragma unroll
    for (int c = 0; c < CPT; ++c) sRed[(g * RT + tr * RPT + a) * (BN + 1) + tc * CPT + c] = acc[a][c];
  __syncthreads();
  double *o = out + ((long long)b * nchunks + chunk) * r * C;
  for (int e = tid; e < RT * BN; e += 256) {
    const int q = e % RT, j = e / RT;
    if (q >= r || c0 + j >= C) continue;
    double s = 0.0;
#pragma unroll
    for (int gg = 0; gg < 4; ++gg) s += (double)sRed[(gg * RT + q) * (BN + 1) + j];
    o[q + (long long)(c0 + j) * r] = s;
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
  const int nct = ceil_div(C, red_bn(C));
  const long long base = (long long)nct * nbatch;
  nchunks = 1;
  if (base < kRedTargetCTAs)
    nchunks = (int)std::min<long long>(ceil_div(kRedTargetCTAs, base), ceil_div(nrows, 256));
  nchunks = std::max(1, nchunks);
  chunk_rows = (int)std::min<long long>(nrows, (long long)ceil_div(ceil_div(nrows, nchunks), kRedBK) * kRedBK);
  nchunks = ceil_div(nrows, chunk_rows);
}

size_t reduce_workspace_doubles(long long nrows, int nbatch, int r, int C, int) {
  int nchunks, chunk_rows;
  reduce_plan(nrows, nbatch, C, nchunks, chunk_rows);
  return nchunks > 1 ? (size_t)nbatch * nchunks * r * C : 0;
}

template <typename T, int RT, int BN>
static cudaError_t reduce_rt(const T *A, long long lda, const T *X, long long ldx, long long nrows, int nbatch,
                             int r, int C, int chunk_rows, int nchunks, int nct, double *dst, const int *skip,
                             cudaStream_t s) {
  const size_t bytes = sizeof(T) * ((size_t)kRedBK * (RT + 1) + (size_t)kRedBK * (BN + 1) + 4ull * RT * (BN + 1));
  auto k = reduce_tn_kernel<T, RT, BN>;
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
  }
  const long long nblk = (long long)nct * nchunks * nbatch;
  HODLR_LAUNCH(k, (unsigned)nblk, 256, bytes, s, A, lda, X, ldx, nrows, r, C, chunk_rows, nchunks, nct, dst, skip);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reduce_tn(const T *A, long long lda, const T *X, long long ldx, long long nrows,
                             int nbatch, int r, int C, double *out, double *work, const int *skip,
                             cudaStream_t s) {
  if (C <= 0 || nbatch <= 0) return cudaSuccess;
  if (r < 1 || r > 64) return cudaErrorInvalidValue;
  int nchunks, chunk_rows;
  reduce_plan(nrows, nbatch, C, nchunks, chunk_rows);
  const int bn = red_bn(C);
  const int nct = ceil_div(C, bn);
  double *dst = nchunks > 1 ? work : out;
  cudaError_t e;
#define HODLR_RED(RTV, BNV) \
  e = reduce_rt<T, RTV, BNV>(A, lda, X, ldx, nrows, nbatch, r, C, chunk_rows, nchunks, nct, dst, skip, s)
  if (bn == 8) {
    if (r <= 16) HODLR_RED(16, 8);
    else if (r <= 32) HODLR_RED(32, 8);
    else HODLR_RED(64, 8);
  } else {
    if (r <= 16) HODLR_RED(16, 64);
    else if (r <= 32) HODLR_RED(32, 64);
    else HODLR_RED(64, 64);
  }
#undef HODLR_RED
  if (e != cudaSuccess) return e;
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
// CTA tile 128 rows x 64 columns, K staged 32 at a time; each thread owns
// rows ti + 16a (a < 8) and columns 4tj .. 4tj+3 (coalesced read-modify-write
// of C along rows).
// The inner dimension is staged BK at a time: 32, or 8 for the rank-k outer
// products of the adjoint (K = nrhs <= 8).
static constexpr int kUpdBM = 128, kUpdBN = 64;

template <typename T, int BK>
__global__ void __launch_bounds__(256) update_nn_kernel(UpdateArgs a, int nrt, int nct) {
  if (a.skip && *a.skip) return;
  __shared__ __align__(16) T sA[BK][kUpdBM];
  __shared__ __align__(16) T sB[BK][kUpdBN + 1];  // +1: conflict-free column stores
  long long lin = blockIdx.x;
  const int rt = (int)(lin % nrt);
  lin /= nrt;
  const int ct = (int)(lin % nct);
  const int b = (int)(lin / nct);
  const int i0 = rt * kUpdBM, j0 = ct * kUpdBN;
  const T *A = reinterpret_cast<const T *>(a.A) + (long long)b * a.a_bstride;
  const double *B = a.B + (long long)(b >> 1) * a.b_s1 + (long long)((b & 1) ^ a.b_flip) * a.b_s2;
  T *C = reinterpret_cast<T *>(a.C) + (long long)b * a.c_bstride;
  const int tid = threadIdx.x, ti = tid & 15, tj = tid >> 4;
  T acc[8][4];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
  for (int q0 = 0; q0 < a.K; q0 += BK) {
    for (int e = tid; e < kUpdBM * BK; e += 256) {
      const int i = e % kUpdBM, q = e / kUpdBM;
      T v = T(0);
      if (i0 + i < a.M && q0 + q < a.K)
        v = a.a_trans ? A[(q0 + q) + (long long)(i0 + i) * a.lda] : A[i0 + i + (long long)(q0 + q) * a.lda];
      sA[q][i] = v;
    }
    for (int e = tid; e < BK * kUpdBN; e += 256) {
      const int q = e % BK, j = e / BK;
      double v = 0.0;
      if (q0 + q < a.K && j0 + j < a.N) {
        v = a.b_trans ? B[(j0 + j) + (long long)(q0 + q) * a.ldb] : B[(q0 + q) + (long long)(j0 + j) * a.ldb];
        if (a.scale) v *= a.scale_cols ? a.scale[j0 + j] : a.scale[q0 + q];
      }
      sB[q][j] = (T)v;
    }
    __syncthreads();
#pragma unroll 4
    for (int q = 0; q < BK; ++q) {
      T av[8], bv[4];
#pragma unroll
      for (int u = 0; u < 8; ++u) av[u] = sA[q][ti + 16 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) bv[v] = sB[q][tj * 4 + v];
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] += av[u] * bv[v];
    }
    __syncthreads();
  }
  const T alpha = (T)a.alpha;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int j = j0 + tj * 4 + v;
    if (j >= a.N) continue;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int i = i0 + ti + 16 * u;
      if (i < a.M) {
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
  if (a.K <= 8)
    HODLR_LAUNCH((update_nn_kernel<T, 8>), (unsigned)nblk, 256, 0, s, a, nrt, nct);
  else
    HODLR_LAUNCH((update_nn_kernel<T, 32>), (unsigned)nblk, 256, 0, s, a, nrt, nct);
  return cudaGetLastError();
}
template cudaError_t launch_update_nn<double>(const UpdateArgs &, cudaStream_t);
template cudaError_t launch_update_nn<float>(const UpdateArgs &, cudaStream_t);

}  // namespace hodlr
