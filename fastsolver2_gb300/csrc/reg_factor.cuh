// Register-resident LU and Gauss-Jordan inverse of one M x M block per CTA
// (M in {32, 64, 128}, 256 threads).
//
// Thread (tx, ty) of a 16 x 16 grid owns the (M/16) x (M/16) tile of rows
// ty*TB.. and columns tx*TB.. in registers for the whole factorisation, so
// each elimination step is TB^2 register FMAs per thread against one column
// and one row broadcast through shared memory -- instead of three shared-
// memory accesses per FMA in a shared-memory-resident elimination.
//
// Pivoting follows LAPACK (first row of maximal |a| in the column, rows
// >= k; netlib_blas/idamax.f:52, dgetf2 semantics).  When the inverse is
// wanted, one Gauss-Jordan sweep produces both: at step k the multipliers
// l_i = a_ik / a_kk (scaled as dgetf2 scales, by the reciprocal unless the
// pivot is tiny) eliminate column k from every other row with the unscaled
// pivot row, so rows >= k see exactly the operations of a right-looking LU
// and the LU factors (row k of U, column k of L) are captured as they appear
// into shared memory, where later row interchanges are applied to the L
// columns already captured (DGETRF's layout); the rows above k carry the
// inverse.  Without the inverse a plain right-looking LU runs.  The inverse
// is written with the column interchanges undone.
#pragma once
#include "dense_ops.cuh"

namespace hodlr {

template <typename T, int TB>
__device__ __forceinline__ T reg_row_select(const T (&a)[TB][TB], int i, int j) {
  T v = a[0][j];
#pragma unroll
  for (int q = 1; q < TB; ++q) v = (q == i) ? a[q][j] : v;
  return v;
}

// Load: functor (i, j) -> T giving the block's entries.  buf: M*M scratch in
// shared memory.  lu_out / ipiv_out / inv_out may be null (skipped).
// *info gets k+1 for the first zero pivot of the LU, else 0.
template <typename T, int M, typename Load, typename StoreInv>
__device__ void reg_factor(Load load, T *buf, T *lu_out, int *ipiv_out, StoreInv store_inv, bool want_inv,
                           int *info) {
  constexpr int TB = M / 16;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  __shared__ T colbuf[M], rowa[M], rowb[M];
  __shared__ int perm[M];
  __shared__ int s_p, s_info;
  T a[TB][TB];
  if (tid == 0) s_info = 0;

  auto fill = [&]() {
    for (int e = tid; e < M * M; e += 256) buf[e] = load(e % M, e / M);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < TB; ++i)
#pragma unroll
      for (int j = 0; j < TB; ++j) a[i][j] = buf[(ty * TB + i) + (tx * TB + j) * M];
    __syncthreads();
  };
  auto stage = [&]() {
#pragma unroll
    for (int i = 0; i < TB; ++i)
#pragma unroll
      for (int j = 0; j < TB; ++j) buf[(ty * TB + i) + (tx * TB + j) * M] = a[i][j];
    __syncthreads();
  };
  // pivot row of column k (values in colbuf), rows >= k; lane 0 publishes s_p
  auto pivot = [&](int k) {
    if (tid < 32) {
      T best = T(-1);
      int bi = -1;
      for (int i = k + tid; i < M; i += 32) {
        const T v = dabs(colbuf[i]);
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
      if (tid == 0) s_p = bi < 0 ? k : bi;
    }
    __syncthreads();
  };
  // swap rows k and p in the register tiles; afterwards rowb holds row k
  auto swap_rows = [&](int kb, int kk, int p) {
    if (p != kb * TB + kk) {
      if (ty == kb)
#pragma unroll
        for (int j = 0; j < TB; ++j) rowa[tx * TB + j] = a[kk][j];
      if (ty == p / TB)
#pragma unroll
        for (int j = 0; j < TB; ++j) rowb[tx * TB + j] = reg_row_select<T, TB>(a, p % TB, j);
      __syncthreads();
      if (ty == kb)
#pragma unroll
        for (int j = 0; j < TB; ++j) a[kk][j] = rowb[tx * TB + j];
      if (ty == p / TB) {
        const int pi = p % TB;
#pragma unroll
        for (int i = 0; i < TB; ++i)
#pragma unroll
          for (int j = 0; j < TB; ++j)
            if (i == pi) a[i][j] = rowa[tx * TB + j];
      }
    } else if (ty == kb) {
#pragma unroll
      for (int j = 0; j < TB; ++j) rowb[tx * TB + j] = a[kk][j];
    }
    __syncthreads();
  };

  // ------------------------------------------------------------- LU
  if (!want_inv && (lu_out || ipiv_out)) {
    fill();
    for (int kb = 0; kb < 16; ++kb) {
#pragma unroll
      for (int kk = 0; kk < TB; ++kk) {
        const int k = kb * TB + kk;
        if (tx == kb)
#pragma unroll
          for (int i = 0; i < TB; ++i) colbuf[ty * TB + i] = a[i][kk];
        __syncthreads();
        pivot(k);
        const int p = s_p;
        if (tid == 0) {
          if (ipiv_out) ipiv_out[k] = p + 1;
          if (colbuf[p] == T(0) && s_info == 0) s_info = k + 1;
        }
        swap_rows(kb, kk, p);
        const T pv = rowb[k];
        if (tx == kb) {
#pragma unroll
          for (int i = 0; i < TB; ++i) {
            const int gi = ty * TB + i;
            if (gi > k && pv != T(0)) a[i][kk] = dabs(pv) >= safe_min<T>() ? a[i][kk] * (T(1) / pv) : a[i][kk] / pv;
            colbuf[gi] = a[i][kk];
          }
        }
        __syncthreads();
        // tiles wholly above or left of the trailing matrix are finished: the
        // threads owning them skip the update (whole warps once k passes their rows)
        if (ty * TB + TB - 1 > k && tx * TB + TB - 1 > k) {
          T cv[TB], rv[TB];
#pragma unroll
          for (int i = 0; i < TB; ++i) cv[i] = colbuf[ty * TB + i];
#pragma unroll
          for (int j = 0; j < TB; ++j) rv[j] = rowb[tx * TB + j];
#pragma unroll
          for (int i = 0; i < TB; ++i)
#pragma unroll
            for (int j = 0; j < TB; ++j)
              if (ty * TB + i > k && tx * TB + j > k) a[i][j] -= cv[i] * rv[j];
        }
        __syncthreads();
      }
    }
    if (lu_out) {
      stage();
      for (int e = tid; e < M * M; e += 256) lu_out[e] = buf[e];
      __syncthreads();
    }
  }
  // ------------------------------------------------------------- Gauss-Jordan
  if (want_inv) {
    const bool capture = lu_out != nullptr;
    fill();  // buf is free from here on: it collects the LU factors
    for (int kb = 0; kb < 16; ++kb) {
#pragma unroll
      for (int kk = 0; kk < TB; ++kk) {
        const int k = kb * TB + kk;
        if (tx == kb)
#pragma unroll
          for (int i = 0; i < TB; ++i) colbuf[ty * TB + i] = a[i][kk];
        __syncthreads();
        pivot(k);
        const int p = s_p;
        if (tid == 0) {
          perm[k] = p;
          if (ipiv_out) ipiv_out[k] = p + 1;
          if (colbuf[p] == T(0) && s_info == 0) s_info = k + 1;
        }
        swap_rows(kb, kk, p);
        // the interchange also applies to the L columns captured so far
        if (capture && p != k)
          for (int j = tid; j < k; j += 256) {
            const T t = buf[k + j * M];
            buf[k + j * M] = buf[p + j * M];
            buf[p + j * M] = t;
          }
        const T pv = rowb[k];
        // multipliers of column k (dgetf2 scaling), captured below the diagonal
        if (tx == kb)
#pragma unroll
          for (int i = 0; i < TB; ++i) {
            const int gi = ty * TB + i;
            T l = a[i][kk];
            if (gi != k && pv != T(0)) l = dabs(pv) >= safe_min<T>() ? l * (T(1) / pv) : l / pv;
            colbuf[gi] = l;
            if (capture && gi > k) buf[gi + k * M] = l;
          }
        if (capture)
          for (int j = k + tid; j < M; j += 256) buf[k + j * M] = rowb[j];  // row k of U
        __syncthreads();
        const T d = pv != T(0) ? T(1) / pv : T(0);
        T cv[TB], rv[TB];
#pragma unroll
        for (int i = 0; i < TB; ++i) cv[i] = colbuf[ty * TB + i];
#pragma unroll
        for (int j = 0; j < TB; ++j) rv[j] = rowb[tx * TB + j];
#pragma unroll
        for (int i = 0; i < TB; ++i) {
          const int gi = ty * TB + i;
#pragma unroll
          for (int j = 0; j < TB; ++j) {
            const int gj = tx * TB + j;
            if (gi == k)
              a[i][j] = (gj == k) ? d : rv[j] * d;
            else
              a[i][j] = (gj == k) ? -cv[i] : a[i][j] - cv[i] * rv[j];
          }
        }
        __syncthreads();
      }
    }
    if (capture) {
      for (int e = tid; e < M * M; e += 256) lu_out[e] = buf[e];
      __syncthreads();
    }
    stage();
    // the row interchanges become column interchanges of the inverse
    if (tid == 0) {
      for (int j = 0; j < M; ++j) colbuf[j] = T(j);
      for (int k = M - 1; k >= 0; --k) {
        const T t = colbuf[k];
        colbuf[k] = colbuf[perm[k]];
        colbuf[perm[k]] = t;
      }
    }
    __syncthreads();
    for (int e = tid; e < M * M; e += 256) {
      const int i = e % M, j = e / M;
      store_inv(i, j, buf[i + (int)colbuf[j] * M]);
    }
    __syncthreads();
  }
  if (tid == 0) *info = s_info;
  __syncthreads();
}

}  // namespace hodlr
