// Block-wide dense LU and triangular solves on one small column-major matrix
// (shared or global memory).  One CTA owns the matrix; all threads of the
// block must call these functions.  These are the per-block arithmetic of
// LAPACK DGETRF / DGETRS (netlib_blas/dgetrf.f, dgetrs.f), reorganised for a
// CTA: warp-shuffle pivot search, 32-row diagonal blocks solved one warp per
// right-hand side, the rest as block-wide multiply-subtracts.
#pragma once
#include <cfloat>

#include "common.cuh"

namespace hodlr {

template <typename T> __device__ __forceinline__ T safe_min();
template <> __device__ __forceinline__ double safe_min<double>() { return DBL_MIN; }
template <> __device__ __forceinline__ float safe_min<float>() { return FLT_MIN; }

template <typename T> __device__ __forceinline__ void swap_vals(T &a, T &b) {
  T t = a;
  a = b;
  b = t;
}

// In-place LU with partial pivoting of the m x m matrix A (lda).  piv gets the
// 1-based LAPACK pivots.  *info = 0, or k+1 for the first zero pivot k.  The
// pivot is the first row of maximal |a| (IDAMAX, netlib_blas/idamax.f:52).
// piv and info may live in shared or global memory.
template <typename T>
__device__ void block_getrf(T *A, int lda, int m, int *piv, int *info) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  __shared__ int s_p;
  __shared__ T s_pv;
  __shared__ int s_info;
  if (tid == 0) s_info = 0;
  const int ti = tid & 31, tj = tid >> 5, ntj = nt >> 5;
  for (int k = 0; k < m; ++k) {
    if (warp == 0) {
      T best = T(-1);
      int bi = -1;
      for (int i = k + lane; i < m; i += 32) {
        T v = dabs(A[i + (long long)k * lda]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        T ob = __shfl_down_sync(0xffffffffu, best, off);
        int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (oi >= 0 && (bi < 0 || ob > best || (ob == best && oi < bi))) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) {
        int p = bi < 0 ? k : bi;
        piv[k] = p + 1;
        s_p = p;
        T pv = A[p + (long long)k * lda];
        s_pv = pv;
        if (pv == T(0) && s_info == 0) s_info = k + 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    const T pv = s_pv;
    if (p != k)
      for (int j = tid; j < m; j += nt) swap_vals(A[k + (long long)j * lda], A[p + (long long)j * lda]);
    __syncthreads();
    if (pv != T(0)) {
      if (dabs(pv) >= safe_min<T>()) {
        const T rcp = T(1) / pv;
        for (int i = k + 1 + tid; i < m; i += nt) A[i + (long long)k * lda] *= rcp;
      } else {
        for (int i = k + 1 + tid; i < m; i += nt) A[i + (long long)k * lda] /= pv;
      }
    }
    __syncthreads();
    for (int j = k + 1 + tj; j < m; j += ntj) {
      const T akj = A[k + (long long)j * lda];
      T *Aj = A + (long long)j * lda;
      const T *Ak = A + (long long)k * lda;
      for (int i = k + 1 + ti; i < m; i += 32) Aj[i] -= Ak[i] * akj;
    }
    __syncthreads();
  }
  if (tid == 0) *info = s_info;
  __syncthreads();
}

// In-place inverse of the n x n matrix A by Gauss-Jordan elimination with
// the partial-pivoting rule of block_getrf (first row of maximal |a|; the
// rows searched are the Schur complement rows, so the pivot sequence is the
// LU's).  Every step is a full 2-D rank-1 update over the block, so all
// threads stay busy: n^3 multiply-adds at 4 block barriers per column.
// fcol: n scratch entries, perm: n ints (shared memory).  Returns the first
// zero pivot (k+1) or 0 in *info.
template <typename T>
__device__ void block_gj_inverse(T *A, int lda, int n, T *fcol, int *perm, int *info) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int ti = tid & 31, tj = tid >> 5, ntj = nt >> 5;
  __shared__ int s_p, s_info;
  if (tid == 0) s_info = 0;
  for (int k = 0; k < n; ++k) {
    if (warp == 0) {
      T best = T(-1);
      int bi = -1;
      for (int i = k + lane; i < n; i += 32) {
        const T v = dabs(A[i + (long long)k * lda]);
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
        perm[k] = p;
        if (A[p + (long long)k * lda] == T(0) && s_info == 0) s_info = k + 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    if (p != k)
      for (int j = tid; j < n; j += nt) swap_vals(A[k + (long long)j * lda], A[p + (long long)j * lda]);
    __syncthreads();
    const T akk = A[k + (long long)k * lda];
    const T d = akk != T(0) ? T(1) / akk : T(0);
    // scale row k (its diagonal becomes d) and save column k
    for (int j = tid; j < n; j += nt) {
      T *x = A + k + (long long)j * lda;
      *x = (j == k) ? d : *x * d;
    }
    for (int i = tid; i < n; i += nt) fcol[i] = A[i + (long long)k * lda];
    __syncthreads();
    for (int j = tj; j < n; j += ntj) {
      const T akj = A[k + (long long)j * lda];
      T *Aj = A + (long long)j * lda;
      for (int i = ti; i < n; i += 32) {
        if (i == k) continue;
        Aj[i] = (j == k) ? -fcol[i] * akj : Aj[i] - fcol[i] * akj;
      }
    }
    __syncthreads();
  }
  // the row interchanges become column interchanges of the inverse, in reverse
  for (int i = tid; i < n; i += nt)
    for (int k = n - 1; k >= 0; --k) {
      const int p = perm[k];
      if (p != k) swap_vals(A[i + (long long)k * lda], A[i + (long long)p * lda]);
    }
  if (tid == 0) *info = s_info;
  __syncthreads();
}

// In-place inverse from the LU factors and pivots of block_getrf, in the
// order of LAPACK DGETRI's unblocked path: inv(U) column by column (DTRTI2),
// then inv(A) inv(L)... solved right to left, then the column interchanges
// undone in reverse.  work: n scratch entries (shared memory).
template <typename T>
__device__ void block_getri(T *A, int lda, int n, const int *piv, T *work) {
  const int tid = threadIdx.x, nt = blockDim.x;
  auto a = [&](int i, int j) -> T & { return A[i + (long long)j * lda]; };
  // 1. inv(U): A[0:j, j] = -inv(U)[j,j] * inv(U)[0:j,0:j] * A[0:j, j]
  for (int j = 0; j < n; ++j) {
    for (int i = tid; i < j; i += nt) work[i] = a(i, j);
    __syncthreads();
    const T dj = T(1) / a(j, j);
    for (int i = tid; i < j; i += nt) {
      T acc = T(0);
      for (int k = i; k < j; ++k) acc += a(i, k) * work[k];
      a(i, j) = -dj * acc;
    }
    __syncthreads();
    if (tid == 0) a(j, j) = dj;
    __syncthreads();
  }
  // 2. solve X L = inv(U) for X, columns n-2 .. 0
  for (int j = n - 2; j >= 0; --j) {
    for (int i = j + 1 + tid; i < n; i += nt) work[i] = a(i, j);
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
      T acc = (i > j) ? T(0) : a(i, j);
      for (int k = j + 1; k < n; ++k) acc -= a(i, k) * work[k];
      a(i, j) = acc;
    }
    __syncthreads();
  }
  // 3. undo the row interchanges of P as column interchanges, in reverse
  for (int i = tid; i < n; i += nt)
    for (int j = n - 2; j >= 0; --j) {
      const int jp = piv[j] - 1;
      if (jp != j) swap_vals(a(i, j), a(i, jp));
    }
  __syncthreads();
}

// Row interchanges of a column tile, in LAPACK DLASWP order (forward) or
// reversed (backward).
template <typename T>
__device__ void block_laswp(const int *piv, int m, T *X, int ldx, int nc, bool forward) {
  for (int j = threadIdx.x; j < nc; j += blockDim.x) {
    T *x = X + (long long)j * ldx;
    if (forward) {
      for (int i = 0; i < m; ++i) {
        int p = piv[i] - 1;
        if (p != i) swap_vals(x[i], x[p]);
      }
    } else {
      for (int i = m - 1; i >= 0; --i) {
        int p = piv[i] - 1;
        if (p != i) swap_vals(x[i], x[p]);
      }
    }
  }
  __syncthreads();
}

// X := A^{-1} X (TRANS = false) or A^{-T} X (TRANS = true) for the LU
// factors LU (lda) and pivots piv of A, X an m x nc tile (ldx).
template <typename T, bool TRANS>
__device__ void block_getrs(const T *LU, int lda, const int *piv, int m, T *X, int ldx, int nc) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  auto lu = [&](int i, int j) -> T { return LU[i + (long long)j * lda]; };
  if (!TRANS) {
    block_laswp(piv, m, X, ldx, nc, true);
    // L y = P b, L unit lower: 32-row blocks, forward
    for (int k0 = 0; k0 < m; k0 += 32) {
      const int kb = min(32, m - k0);
      for (int j = warp; j < nc; j += nwarp) {
        T *x = X + (long long)j * ldx + k0;
        T v = lane < kb ? x[lane] : T(0);
        for (int kk = 0; kk < kb - 1; ++kk) {
          T xk = __shfl_sync(0xffffffffu, v, kk);
          if (lane > kk && lane < kb) v -= lu(k0 + lane, k0 + kk) * xk;
        }
        if (lane < kb) x[lane] = v;
      }
      __syncthreads();
      const int rows = m - k0 - kb;
      if (rows > 0) {
        for (int e = tid; e < rows * nc; e += nt) {
          const int i = k0 + kb + e % rows, j = e / rows;
          T *x = X + (long long)j * ldx;
          T acc = x[i];
          for (int kk = 0; kk < kb; ++kk) acc -= lu(i, k0 + kk) * x[k0 + kk];
          x[i] = acc;
        }
      }
      __syncthreads();
    }
    // U x = y, U non-unit upper: 32-row blocks, backward
    for (int k1 = m; k1 > 0; k1 -= 32) {
      const int k0 = max(0, k1 - 32), kb = k1 - k0;
      for (int j = warp; j < nc; j += nwarp) {
        T *x = X + (long long)j * ldx + k0;
        T v = lane < kb ? x[lane] : T(0);
        for (int kk = kb - 1; kk >= 0; --kk) {
          if (lane == kk) v = v / lu(k0 + kk, k0 + kk);
          T xk = __shfl_sync(0xffffffffu, v, kk);
          if (lane < kk) v -= lu(k0 + lane, k0 + kk) * xk;
        }
        if (lane < kb) x[lane] = v;
      }
      __syncthreads();
      if (k0 > 0) {
        for (int e = tid; e < k0 * nc; e += nt) {
          const int i = e % k0, j = e / k0;
          T *x = X + (long long)j * ldx;
          T acc = x[i];
          for (int kk = 0; kk < kb; ++kk) acc -= lu(i, k0 + kk) * x[k0 + kk];
          x[i] = acc;
        }
      }
      __syncthreads();
    }
  } else {
    // U^T y = b, U^T non-unit lower: forward
    for (int k0 = 0; k0 < m; k0 += 32) {
      const int kb = min(32, m - k0);
      for (int j = warp; j < nc; j += nwarp) {
        T *x = X + (long long)j * ldx + k0;
        T v = lane < kb ? x[lane] : T(0);
        for (int kk = 0; kk < kb; ++kk) {
          if (lane == kk) v = v / lu(k0 + kk, k0 + kk);
          T xk = __shfl_sync(0xffffffffu, v, kk);
          if (lane > kk && lane < kb) v -= lu(k0 + kk, k0 + lane) * xk;
        }
        if (lane < kb) x[lane] = v;
      }
      __syncthreads();
      const int rows = m - k0 - kb;
      if (rows > 0) {
        for (int e = tid; e < rows * nc; e += nt) {
          const int i = k0 + kb + e % rows, j = e / rows;
          T *x = X + (long long)j * ldx;
          T acc = x[i];
          for (int kk = 0; kk < kb; ++kk) acc -= lu(k0 + kk, i) * x[k0 + kk];
          x[i] = acc;
        }
      }
      __syncthreads();
    }
    // L^T z = y, L^T unit upper: backward
    for (int k1 = m; k1 > 0; k1 -= 32) {
      const int k0 = max(0, k1 - 32), kb = k1 - k0;
      for (int j = warp; j < nc; j += nwarp) {
        T *x = X + (long long)j * ldx + k0;
        T v = lane < kb ? x[lane] : T(0);
        for (int kk = kb - 1; kk > 0; --kk) {
          T xk = __shfl_sync(0xffffffffu, v, kk);
          if (lane < kk) v -= lu(k0 + kk, k0 + lane) * xk;
        }
        if (lane < kb) x[lane] = v;
      }
      __syncthreads();
      if (k0 > 0) {
        for (int e = tid; e < k0 * nc; e += nt) {
          const int i = e % k0, j = e / k0;
          T *x = X + (long long)j * ldx;
          T acc = x[i];
          for (int kk = 0; kk < kb; ++kk) acc -= lu(k0 + kk, i) * x[k0 + kk];
          x[i] = acc;
        }
      }
      __syncthreads();
    }
    block_laswp(piv, m, X, ldx, nc, false);
  }
}

}  // namespace hodlr
