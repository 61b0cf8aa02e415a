// K1 / K2: batched leaf LU and leaf triangular solves.
//
// Replaces the leaf case of fastSolver2's hsolve, one dgesv per leaf on the
// CPU (src/tasks/leaf_solve.cc:80-92): here every leaf of the tree is
// factorised by one launch (one CTA per leaf, the block staged in shared
// memory when it fits) and the solves against all right-hand-side columns
// are one launch over (leaf, column tile).
#include <algorithm>

#include "dense_ops.cuh"
#include "kernels.cuh"
#include "reg_factor.cuh"

namespace hodlr {

template <typename T, bool SMEM>
__global__ void __launch_bounds__(256)
leaf_getrf_kernel(const double *__restrict__ D, long long d_ld, long long d_stride, T *LU, int *ipiv,
                  int m, DevStatus *st, T *Dinv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_bad;
  __shared__ int s_info;
  const int leaf = blockIdx.x;
  const double *Dg = D + (long long)leaf * d_stride;
  T *LUg = LU + (long long)leaf * m * m;
  T *A = SMEM ? reinterpret_cast<T *>(smem_raw) : LUg;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  int bad = 0;
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int i = e % m, j = e / m;
    const double v = Dg[i + (long long)j * d_ld];
    if (!isfinite(v)) bad = 1;
    A[e] = (T)v;
  }
  if (bad) atomicOr(&s_bad, 1);
  __syncthreads();
  if (s_bad) {
    if (threadIdx.x == 0) report_error(st, HODLR_ERR_NONFINITE_INPUT, (long long)leaf * m);
    return;
  }
  block_getrf<T>(A, m, m, ipiv + (long long)leaf * m, &s_info);
  if (s_info && threadIdx.x == 0) report_error(st, HODLR_ERR_SINGULAR_LEAF, leaf);
  if (SMEM) {
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) LUg[e] = A[e];
    if (Dinv) {  // explicit inverse: Gauss-Jordan on a fresh copy of the block
      __syncthreads();
      for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
        const int i = e % m, j = e / m;
        A[e] = (T)Dg[i + (long long)j * d_ld];
      }
      __syncthreads();
      T *fcol = A + (size_t)m * m;
      int *perm = reinterpret_cast<int *>(fcol + m);
      block_gj_inverse<T>(A, m, m, fcol, perm, &s_info);
      T *out = Dinv + (long long)leaf * m * m;
      for (int e = threadIdx.x; e < m * m; e += blockDim.x) out[e] = A[e];
    }
  }
}

// Leaf LU (+ optional explicit inverse) with the block resident in registers
// (reg_factor.cuh), for M in {32, 64, 128}.
template <typename T, int M>
__global__ void __launch_bounds__(256, (sizeof(T) == 4 && M == 128) ? 2 : 1)
leaf_factor_reg_kernel(const double *__restrict__ D, long long d_ld, long long d_stride, T *LU, int *ipiv,
                       DevStatus *st, T *Dinv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_bad, s_info;
  T *buf = reinterpret_cast<T *>(smem_raw);
  const int leaf = blockIdx.x;
  const double *Dg = D + (long long)leaf * d_stride;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  int bad = 0;
  for (int e = threadIdx.x; e < M * M; e += blockDim.x)
    if (!isfinite(Dg[(e % M) + (long long)(e / M) * d_ld])) bad = 1;
  if (bad) atomicOr(&s_bad, 1);
  __syncthreads();
  if (s_bad) {
    if (threadIdx.x == 0) report_error(st, HODLR_ERR_NONFINITE_INPUT, (long long)leaf * M);
    return;
  }
  T *inv = Dinv ? Dinv + (long long)leaf * M * M : nullptr;
  auto load = [&](int i, int j) -> T { return (T)Dg[i + (long long)j * d_ld]; };
  auto store = [&](int i, int j, T v) { inv[i + j * M] = v; };
  reg_factor<T, M>(load, buf, LU + (long long)leaf * M * M, ipiv + (long long)leaf * M, store, inv != nullptr,
                   &s_info);
  if (s_info && threadIdx.x == 0) report_error(st, HODLR_ERR_SINGULAR_LEAF, leaf);
}

template <typename T, bool TRANS, bool LU_SMEM>
__global__ void __launch_bounds__(256)
leaf_getrs_kernel(const T *__restrict__ LU, const int *__restrict__ ipiv, int m, T *X, long long ldx,
                  int ncols, int ct, const int *skip) {
  if (skip && *skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int leaf = blockIdx.y;
  const int c0 = blockIdx.x * ct;
  const int nc = min(ct, ncols - c0);
  T *sX = reinterpret_cast<T *>(smem_raw);
  int *spiv = reinterpret_cast<int *>(sX + (size_t)m * ct);
  T *sLU = reinterpret_cast<T *>(reinterpret_cast<uintptr_t>(spiv + m + 3) & ~uintptr_t(15));
  const T *gLU = LU + (long long)leaf * m * m;
  for (int i = threadIdx.x; i < m; i += blockDim.x) spiv[i] = ipiv[(long long)leaf * m + i];
  if (LU_SMEM)
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) sLU[e] = gLU[e];
  T *Xg = X + (long long)leaf * m + (long long)c0 * ldx;
  for (int e = threadIdx.x; e < m * nc; e += blockDim.x) {
    const int i = e % m, j = e / m;
    sX[e] = Xg[i + (long long)j * ldx];
  }
  __syncthreads();
  block_getrs<T, TRANS>(LU_SMEM ? sLU : gLU, m, spiv, m, sX, m, nc);
  for (int e = threadIdx.x; e < m * nc; e += blockDim.x) {
    const int i = e % m, j = e / m;
    Xg[i + (long long)j * ldx] = sX[e];
  }
}

static constexpr size_t kSmemCap = 220 * 1024;

template <typename K>
static cudaError_t set_smem(K kernel, size_t bytes) {
  return allow_dyn_smem(kernel, bytes);
}

static bool reg_leaf(int m) { return m == 32 || m == 64 || m == 128; }

bool leaf_getrf_fused_inverse(int m, int elem_bytes) {
  return reg_leaf(m) || (size_t)m * (m + 1) * elem_bytes + (size_t)m * 4 <= kSmemCap;
}

template <typename T, int M>
static cudaError_t launch_reg(const double *D, long long d_ld, long long d_stride, T *LU, int *ipiv, int nleaf,
                              DevStatus *st, T *Dinv, cudaStream_t s) {
  const size_t bytes = (size_t)M * M * sizeof(T);
  auto k = leaf_factor_reg_kernel<T, M>;
  cudaError_t e = set_smem(k, bytes);
  if (e != cudaSuccess) return e;
  HODLR_LAUNCH(k, nleaf, 256, bytes, s, D, d_ld, d_stride, LU, ipiv, st, Dinv);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_leaf_getrf(const double *D, long long d_ld, long long d_stride, T *LU, int *ipiv,
                              int m, int nleaf, DevStatus *st, T *Dinv, cudaStream_t s) {
  if (m == 32) return launch_reg<T, 32>(D, d_ld, d_stride, LU, ipiv, nleaf, st, Dinv, s);
  if (m == 64) return launch_reg<T, 64>(D, d_ld, d_stride, LU, ipiv, nleaf, st, Dinv, s);
  if (m == 128) return launch_reg<T, 128>(D, d_ld, d_stride, LU, ipiv, nleaf, st, Dinv, s);
  const size_t bytes = (size_t)m * (m + 1) * sizeof(T) + (size_t)m * 4;
  if (bytes <= kSmemCap) {
    auto k = leaf_getrf_kernel<T, true>;
    cudaError_t e = set_smem(k, bytes);
    if (e != cudaSuccess) return e;
    HODLR_LAUNCH(k, nleaf, 256, bytes, s, D, d_ld, d_stride, LU, ipiv, m, st, Dinv);
  } else {
    if (Dinv) return cudaErrorInvalidValue;  // caller forms the inverse separately
    return launch_leaf_getrf_blocked<T>(D, d_ld, d_stride, LU, ipiv, m, nleaf, st, s);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_leaf_getrs(const T *LU, const int *ipiv, int m, int nleaf, T *X, long long ldx,
                              int ncols, bool trans, const int *skip, cudaStream_t s) {
  if (ncols <= 0 || nleaf <= 0) return cudaSuccess;
  const size_t lu_bytes = (size_t)m * m * sizeof(T);
  const size_t piv_bytes = (size_t)m * sizeof(int) + 16;
  // FP32: keep two CTAs per SM; FP64 is DFMA-bound, one CTA per SM suffices.
  const size_t cap = sizeof(T) == 4 ? 110 * 1024 : kSmemCap;
  bool lu_smem = lu_bytes + piv_bytes + (size_t)m * 8 * sizeof(T) <= cap;
  size_t avail = cap - piv_bytes - (lu_smem ? lu_bytes : 0);
  int ct_max = (int)std::min<size_t>(avail / ((size_t)m * sizeof(T)), 128);
  if (ct_max < 1) return cudaErrorInvalidValue;
  // enough column tiles to give every SM a CTA when the leaves are few and large
  int ntile = std::max(ceil_div(ncols, ct_max), std::min(ncols, ceil_div(kNumSMs, nleaf)));
  int ct = ceil_div(ncols, ntile);
  ntile = ceil_div(ncols, ct);
  size_t bytes = (size_t)m * ct * sizeof(T) + piv_bytes + (lu_smem ? lu_bytes : 0);
  dim3 grid(ntile, nleaf);
  cudaError_t e = cudaSuccess;
#define HODLR_GETRS_CASE(TR, LS)                                                     \
  {                                                                                  \
    auto k = leaf_getrs_kernel<T, TR, LS>;                                           \
    e = set_smem(k, bytes);                                                          \
    if (e != cudaSuccess) return e;                                                  \
    HODLR_LAUNCH(k, grid, 256, bytes, s, LU, ipiv, m, X, ldx, ncols, ct, skip);      \
  }
  if (!trans) {
    if (lu_smem) HODLR_GETRS_CASE(false, true) else HODLR_GETRS_CASE(false, false)
  } else {
    if (lu_smem) HODLR_GETRS_CASE(true, true) else HODLR_GETRS_CASE(true, false)
  }
#undef HODLR_GETRS_CASE
  return cudaGetLastError();
}

template cudaError_t launch_leaf_getrf<double>(const double *, long long, long long, double *, int *, int,
                                               int, DevStatus *, double *, cudaStream_t);
template cudaError_t launch_leaf_getrf<float>(const double *, long long, long long, float *, int *, int,
                                              int, DevStatus *, float *, cudaStream_t);
template cudaError_t launch_leaf_getrs<double>(const double *, const int *, int, int, double *, long long,
                                               int, bool, const int *, cudaStream_t);
template cudaError_t launch_leaf_getrs<float>(const float *, const int *, int, int, float *, long long, int,
                                              bool, const int *, cudaStream_t);

}  // namespace hodlr
