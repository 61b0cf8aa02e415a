// K1 for leaves too large for one CTA's shared memory: batched right-looking
// blocked LU, the blocked order of LAPACK DGETRF (netlib_blas/dgetrf.f:109 --
// factor a panel of nb columns, apply its interchanges to the other columns
// (DLASWP), U12 = L11^{-1} A12 (DTRSM), A22 -= L21 U12 (DGEMM)), here with the
// panel of every leaf factored by one CTA in shared memory and the triangular
// solve and trailing update of every leaf spread over (column tile, leaf)
// CTAs, so the whole GPU works on a few large leaves.
//
// The result has the layout of the one-CTA kernels: LU [nleaf][m][m]
// column-major with the unit lower factor below the diagonal, 1-based pivots
// [nleaf][m], the first zero pivot reported as HODLR_ERR_SINGULAR_LEAF.
#include <algorithm>

#include "dense_ops.cuh"
#include "kernels.cuh"

namespace hodlr {

constexpr int kPanelNb = 32;      // panel width
constexpr int kTrailCols = 32;    // columns per trailing-update CTA
constexpr int kTrailRows = 128;   // rows of L21 staged per pass

template <typename T>
static cudaError_t set_dyn_smem(T kernel, size_t bytes) {
  return allow_dyn_smem(kernel, bytes);
}

// LU[leaf] = (T) D[leaf]; the first non-finite entry is reported.
template <typename T>
__global__ void __launch_bounds__(256) leaf_blocked_init_kernel(const double *__restrict__ D, long long d_ld,
                                                                long long d_stride, int m, T *LU, DevStatus *st) {
  const int leaf = blockIdx.y;
  const double *Dg = D + (long long)leaf * d_stride;
  T *A = LU + (long long)leaf * m * m;
  const long long mm = (long long)m * m;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < mm; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % m), j = (int)(e / m);
    const double v = Dg[i + (long long)j * d_ld];
    if (!isfinite(v)) report_error(st, HODLR_ERR_NONFINITE_INPUT, (long long)leaf * m);
    A[e] = (T)v;
  }
}

// Panel [j0, j0 + jb) of every leaf (one CTA each): LU with partial pivoting
// of rows [j0, m) (the pivot is the first row of largest |a|, IDAMAX; the
// column under it scaled by the pivot's reciprocal), staged in shared memory
// when `staged`; then the panel's interchanges applied to every other column.
template <typename T>
__global__ void __launch_bounds__(256) leaf_panel_kernel(T *LU, int m, int j0, int jb, int *ipiv, int staged,
                                                         DevStatus *st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_p, s_info, s_piv[kPanelNb];
  __shared__ T s_pv;
  const int leaf = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
  T *A = LU + (long long)leaf * m * m;
  const int rows = m - j0;
  T *P = staged ? reinterpret_cast<T *>(smem_raw) : A + j0 + (long long)j0 * m;
  const long long ldp = staged ? rows : m;
  if (tid == 0) s_info = 0;
  if (staged)
    for (int e = tid; e < rows * jb; e += nt) {
      const int i = e % rows, j = e / rows;
      P[e] = A[(j0 + i) + (long long)(j0 + j) * m];
    }
  __syncthreads();
  for (int k = 0; k < jb; ++k) {
    if (warp == 0) {
      T best = T(-1);
      int bi = -1;
      for (int i = k + lane; i < rows; i += 32) {
        const T v = dabs(P[i + k * ldp]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        const T ob = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (oi >= 0 && (bi < 0 || ob > best || (ob == best && oi < bi))) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) {
        const int p = bi < 0 ? k : bi;
        s_p = p;
        s_piv[k] = j0 + p;
        s_pv = P[p + k * ldp];
        if (s_pv == T(0) && s_info == 0) s_info = j0 + k + 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    const T pv = s_pv;
    if (p != k)
      for (int j = tid; j < jb; j += nt) swap_vals(P[k + j * ldp], P[p + j * ldp]);
    __syncthreads();
    if (pv != T(0)) {
      if (dabs(pv) >= safe_min<T>()) {
        const T rcp = T(1) / pv;
        for (int i = k + 1 + tid; i < rows; i += nt) P[i + k * ldp] *= rcp;
      } else {
        for (int i = k + 1 + tid; i < rows; i += nt) P[i + k * ldp] /= pv;
      }
    }
    __syncthreads();
    const int nj = jb - k - 1;
    for (int e = tid; e < (rows - k - 1) * nj; e += nt) {
      const int i = k + 1 + e % (rows - k - 1), j = k + 1 + e / (rows - k - 1);
      P[i + j * ldp] -= P[i + k * ldp] * P[k + j * ldp];
    }
    __syncthreads();
  }
  if (staged)
    for (int e = tid; e < rows * jb; e += nt) {
      const int i = e % rows, j = e / rows;
      A[(j0 + i) + (long long)(j0 + j) * m] = P[e];
    }
  for (int k = tid; k < jb; k += nt) ipiv[(long long)leaf * m + j0 + k] = s_piv[k] + 1;
  // the interchanges on the columns left and right of the panel, one thread per column
  for (int c = tid; c < m - jb; c += nt) {
    const int col = c < j0 ? c : c + jb;
    T *Ac = A + (long long)col * m;
    for (int k = 0; k < jb; ++k) {
      const int p = s_piv[k];
      if (p != j0 + k) swap_vals(Ac[j0 + k], Ac[p]);
    }
  }
  if (tid == 0 && s_info) report_error(st, HODLR_ERR_SINGULAR_LEAF, leaf);
}

// Trailing update after panel [j0, j0 + jb): CTA (tile, leaf) owns columns
// [c0, c0 + 32) right of the panel: U12 = L11^{-1} A12 (unit lower, column
// by column in DTRSM's order), then A22 -= L21 U12 in passes of 128 rows, the
// products of each entry summed in panel-column order.
template <typename T>
__global__ void __launch_bounds__(256) leaf_trail_kernel(T *LU, int m, int j0, int jb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sL11 = reinterpret_cast<T *>(smem_raw);          // jb x jb, ld kPanelNb
  T *sU = sL11 + kPanelNb * kPanelNb;                 // jb x 32, ld kPanelNb
  T *sL21 = sU + kPanelNb * kTrailCols;               // 128 x jb, element (r, k) at [k * 128 + r]
  const int leaf = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  T *A = LU + (long long)leaf * m * m;
  const int c0 = j0 + jb + blockIdx.x * kTrailCols;
  const int nc = min(kTrailCols, m - c0);
  for (int e = tid; e < jb * jb; e += nt) {
    const int i = e % jb, k = e / jb;
    sL11[i + k * kPanelNb] = A[(j0 + i) + (long long)(j0 + k) * m];
  }
  for (int e = tid; e < jb * nc; e += nt) {
    const int i = e % jb, c = e / jb;
    sU[i + c * kPanelNb] = A[(j0 + i) + (long long)(c0 + c) * m];
  }
  __syncthreads();
  // U12: k-th step subtracts x_k L11(i, k) from the rows below k, all columns at once
  for (int k = 0; k + 1 < jb; ++k) {
    for (int e = tid; e < (jb - k - 1) * nc; e += nt) {
      const int i = k + 1 + e % (jb - k - 1), c = e / (jb - k - 1);
      sU[i + c * kPanelNb] -= sU[k + c * kPanelNb] * sL11[i + k * kPanelNb];
    }
    __syncthreads();
  }
  for (int e = tid; e < jb * nc; e += nt) {
    const int i = e % jb, c = e / jb;
    A[(j0 + i) + (long long)(c0 + c) * m] = sU[i + c * kPanelNb];
  }
  // A22 -= L21 U12: thread (lane, group) owns rows lane + 32a (a < 4) and columns 4 group + b (b < 4)
  const int lane = tid & 31, grp = tid >> 5;
  for (int r0 = j0 + jb; r0 < m; r0 += kTrailRows) {
    const int nr = min(kTrailRows, m - r0);
    __syncthreads();
    for (int e = tid; e < kTrailRows * jb; e += nt) {
      const int r = e % kTrailRows, k = e / kTrailRows;
      sL21[k * kTrailRows + r] = r < nr ? A[(r0 + r) + (long long)(j0 + k) * m] : T(0);
    }
    __syncthreads();
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int r = lane + 32 * a, c = 4 * grp + b;
        acc[a][b] = (r < nr && c < nc) ? A[(r0 + r) + (long long)(c0 + c) * m] : T(0);
      }
    for (int k = 0; k < jb; ++k) {
      T l[4], u[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) l[a] = sL21[k * kTrailRows + lane + 32 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) u[b] = sU[k + (4 * grp + b) * kPanelNb];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] -= l[a] * u[b];
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int r = lane + 32 * a, c = 4 * grp + b;
        if (r < nr && c < nc) A[(r0 + r) + (long long)(c0 + c) * m] = acc[a][b];
      }
  }
}

// Explicit inverses D^{-1} = U^{-1} L^{-1} P from the LU factors of every leaf:
// CTA (tile, leaf) owns columns [c0, c0 + 32) of the inverse, all m rows in
// shared memory.  The identity's columns get the interchanges, then a blocked
// unit-lower solve (32-row diagonal blocks in DTRSM's order, the rows below
// updated by the block's L panel in passes of 128 rows) and a blocked upper
// solve from the bottom (diagonal blocks by division, the rows above updated
// by the block's U panel) -- the DGETRS order on the identity.  (For solves
// with a few right-hand sides the one-CTA-per-column-tile kernel of
// launch_leaf_getrs, which spreads the columns over every SM, is faster.)
template <typename T>
__global__ void __launch_bounds__(256) leaf_inverse_blocked_kernel(const T *__restrict__ LU,
                                                                   const int *__restrict__ ipiv, int m, T *Dinv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sX = reinterpret_cast<T *>(smem_raw);                 // m x 32, ld m
  T *sP = sX + (size_t)m * kTrailCols;                      // panel pass: 128 x 32, [k * 128 + r]
  T *sD = sP + kTrailRows * kPanelNb;                       // diagonal block 32 x 32, ld 32
  const int leaf = blockIdx.y, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, grp = tid >> 5;
  const T *A = LU + (long long)leaf * m * m;
  const int *piv = ipiv + (long long)leaf * m;
  const int c0 = blockIdx.x * kTrailCols, nc = min(kTrailCols, m - c0);
  T *out = Dinv + (long long)leaf * m * m + (long long)c0 * m;
  for (int e = tid; e < m * kTrailCols; e += nt) {
    const int i = e % m, c = e / m;
    sX[e] = (c < nc && i == c0 + c) ? T(1) : T(0);
  }
  __syncthreads();
  if (tid < nc)
    for (int k = 0; k < m; ++k) {
      const int p = piv[k] - 1;
      if (p != k) swap_vals(sX[k + tid * m], sX[p + tid * m]);
    }
  // rows [r0, r0 + nr) -= A(rows, kb block) * X(kb block rows, :), the panel streamed in 128-row passes
  auto panel_update = [&](int kb0, int kbn, int r0, int r1) {
    for (int p0 = r0; p0 < r1; p0 += kTrailRows) {
      const int nr = min(kTrailRows, r1 - p0);
      __syncthreads();
      for (int e = tid; e < kTrailRows * kbn; e += nt) {
        const int r = e % kTrailRows, k = e / kTrailRows;
        sP[k * kTrailRows + r] = r < nr ? A[(p0 + r) + (long long)(kb0 + k) * m] : T(0);
      }
      __syncthreads();
      T acc[4][4];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int r = lane + 32 * a;
          acc[a][b] = r < nr ? sX[(p0 + r) + (4 * grp + b) * m] : T(0);
        }
      for (int k = 0; k < kbn; ++k) {
        T l[4], u[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) l[a] = sP[k * kTrailRows + lane + 32 * a];
#pragma unroll
        for (int b = 0; b < 4; ++b) u[b] = sX[(kb0 + k) + (4 * grp + b) * m];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] -= l[a] * u[b];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int r = lane + 32 * a;
          if (r < nr) sX[(p0 + r) + (4 * grp + b) * m] = acc[a][b];
        }
    }
  };
  auto load_diag = [&](int kb0, int kbn) {
    __syncthreads();
    for (int e = tid; e < kbn * kbn; e += nt) {
      const int i = e % kbn, k = e / kbn;
      sD[i + k * kPanelNb] = A[(kb0 + i) + (long long)(kb0 + k) * m];
    }
    __syncthreads();
  };
  // L Y = P X, unit lower, 32-row blocks top down
  for (int kb0 = 0; kb0 < m; kb0 += kPanelNb) {
    const int kbn = min(kPanelNb, m - kb0);
    load_diag(kb0, kbn);
    for (int k = 0; k + 1 < kbn; ++k) {
      for (int e = tid; e < (kbn - k - 1) * kTrailCols; e += nt) {
        const int i = k + 1 + e % (kbn - k - 1), c = e / (kbn - k - 1);
        sX[(kb0 + i) + c * m] -= sX[(kb0 + k) + c * m] * sD[i + k * kPanelNb];
      }
      __syncthreads();
    }
    if (kb0 + kbn < m) panel_update(kb0, kbn, kb0 + kbn, m);
  }
  // U X = Y, 32-row blocks bottom up
  for (int kb0 = ((m - 1) / kPanelNb) * kPanelNb; kb0 >= 0; kb0 -= kPanelNb) {
    const int kbn = min(kPanelNb, m - kb0);
    load_diag(kb0, kbn);
    for (int k = kbn - 1; k >= 0; --k) {
      if (tid < kTrailCols) sX[(kb0 + k) + tid * m] /= sD[k + k * kPanelNb];
      __syncthreads();
      for (int e = tid; e < k * kTrailCols; e += nt) {
        const int i = e % k, c = e / k;
        sX[(kb0 + i) + c * m] -= sX[(kb0 + k) + c * m] * sD[i + k * kPanelNb];
      }
      __syncthreads();
    }
    if (kb0 > 0) panel_update(kb0, kbn, 0, kb0);
  }
  __syncthreads();
  for (int e = tid; e < m * nc; e += nt) {
    const int i = e % m, c = e / m;
    out[i + (long long)c * m] = sX[i + c * m];
  }
}

size_t leaf_inverse_blocked_smem(int m, int elem_bytes) {
  return (size_t)elem_bytes * ((size_t)m * kTrailCols + (size_t)kTrailRows * kPanelNb + (size_t)kPanelNb * kPanelNb);
}

template <typename T>
cudaError_t launch_leaf_inverse_blocked(const T *LU, const int *ipiv, int m, int nleaf, T *Dinv, cudaStream_t s) {
  const size_t bytes = leaf_inverse_blocked_smem(m, sizeof(T));
  cudaError_t e = set_dyn_smem(leaf_inverse_blocked_kernel<T>, bytes);
  if (e != cudaSuccess) return e;
  dim3 grid(ceil_div(m, kTrailCols), nleaf);
  HODLR_LAUNCH(leaf_inverse_blocked_kernel<T>, grid, 256, bytes, s, LU, ipiv, m, Dinv);
  return cudaGetLastError();
}

template cudaError_t launch_leaf_inverse_blocked<double>(const double *, const int *, int, int, double *,
                                                         cudaStream_t);
template cudaError_t launch_leaf_inverse_blocked<float>(const float *, const int *, int, int, float *, cudaStream_t);


template <typename T>
cudaError_t launch_leaf_getrf_blocked(const double *D, long long d_ld, long long d_stride, T *LU, int *ipiv, int m,
                                      int nleaf, DevStatus *st, cudaStream_t s) {
  if (m < 1 || nleaf < 1) return cudaSuccess;
  {
    const long long per = ((long long)m * m + 255) / 256;
    dim3 grid((unsigned)std::min<long long>(per, 64), nleaf);
    HODLR_LAUNCH(leaf_blocked_init_kernel<T>, grid, 256, 0, s, D, d_ld, d_stride, m, LU, st);
  }
  const size_t trail_bytes = sizeof(T) * ((size_t)kPanelNb * kPanelNb + (size_t)kPanelNb * kTrailCols +
                                          (size_t)kTrailRows * kPanelNb);
  cudaError_t e = set_dyn_smem(leaf_trail_kernel<T>, trail_bytes);
  if (e != cudaSuccess) return e;
  constexpr size_t kPanelSmemCap = 200 * 1024;
  for (int j0 = 0; j0 < m; j0 += kPanelNb) {
    const int jb = std::min(kPanelNb, m - j0);
    const size_t pbytes = sizeof(T) * (size_t)(m - j0) * jb;
    const bool staged = pbytes <= kPanelSmemCap;
    if (staged) {
      e = set_dyn_smem(leaf_panel_kernel<T>, pbytes);
      if (e != cudaSuccess) return e;
    }
    HODLR_LAUNCH(leaf_panel_kernel<T>, nleaf, 256, staged ? pbytes : 0, s, LU, m, j0, jb, ipiv, (int)staged, st);
    const int rest = m - j0 - jb;
    if (rest > 0) {
      dim3 grid(ceil_div(rest, kTrailCols), nleaf);
      HODLR_LAUNCH(leaf_trail_kernel<T>, grid, 256, trail_bytes, s, LU, m, j0, jb);
    }
  }
  return cudaGetLastError();
}

template cudaError_t launch_leaf_getrf_blocked<double>(const double *, long long, long long, double *, int *, int,
                                                       int, DevStatus *, cudaStream_t);
template cudaError_t launch_leaf_getrf_blocked<float>(const double *, long long, long long, float *, int *, int,
                                                      int, DevStatus *, cudaStream_t);

}  // namespace hodlr
