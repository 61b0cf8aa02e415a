// Explicit-inverse application kernels.
//
// The small dense systems of the sweep (leaf blocks, m x m; capacitance
// systems, 2r x 2r) are factorised once with partial pivoting (LU, as the
// reference's dgesv calls do, src/tasks/leaf_solve.cc:89,140) and their
// inverses A^{-1} = U^{-1} L^{-1} P are formed from the LU factors in the
// same factorisation pass.  Every later application -- to the L*r columns of
// the transformed bases, to the right-hand sides of each solve and of every
// refinement step -- is then a batched GEMM instead of a pair of triangular
// solves: no per-row synchronisation, full register tiling, and the same
// flop count as the two triangular solves it replaces.
#include <algorithm>
#include <type_traits>

#include "dense_ops.cuh"
#include "kernels.cuh"
#include "reg_factor.cuh"
#include "resid_emul.cuh"

namespace hodlr {

static constexpr size_t kSmemCap = 220 * 1024;

template <typename K>
static cudaError_t set_smem(K kernel, size_t bytes) {
  return allow_dyn_smem(kernel, bytes);
}

// --------------------------------------------------------- leaf inverse
// Dinv_i = D_i^{-1} from the stored LU factors: getrs against identity
// column tiles.  grid (tiles, nleaf).
template <typename T, bool LU_SMEM>
__global__ void __launch_bounds__(256)
leaf_inverse_kernel(const T *__restrict__ LU, const int *__restrict__ ipiv, int m, T *Dinv, int ct) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int leaf = blockIdx.y, c0 = blockIdx.x * ct, nc = min(ct, m - c0);
  T *sX = reinterpret_cast<T *>(smem_raw);
  int *spiv = reinterpret_cast<int *>(sX + (size_t)m * ct);
  T *sLU = reinterpret_cast<T *>(reinterpret_cast<uintptr_t>(spiv + m + 3) & ~uintptr_t(15));
  const T *gLU = LU + (long long)leaf * m * m;
  for (int i = threadIdx.x; i < m; i += blockDim.x) spiv[i] = ipiv[(long long)leaf * m + i];
  if (LU_SMEM)
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) sLU[e] = gLU[e];
  for (int e = threadIdx.x; e < m * nc; e += blockDim.x) {
    const int i = e % m, j = e / m;
    sX[e] = (i == c0 + j) ? T(1) : T(0);
  }
  __syncthreads();
  block_getrs<T, false>(LU_SMEM ? sLU : gLU, m, spiv, m, sX, m, nc);
  T *out = Dinv + (long long)leaf * m * m + (long long)c0 * m;
  for (int e = threadIdx.x; e < m * nc; e += blockDim.x) out[e] = sX[e];
}

template <typename T>
cudaError_t launch_leaf_inverse(const T *LU, const int *ipiv, int m, int nleaf, T *Dinv, cudaStream_t s) {
  const size_t lu_bytes = (size_t)m * m * sizeof(T), piv_bytes = (size_t)m * 4 + 16;
  const bool lu_smem = lu_bytes + piv_bytes + (size_t)m * 8 * sizeof(T) <= kSmemCap;
  if (!lu_smem && leaf_inverse_blocked_smem(m, sizeof(T)) <= kSmemCap)
    return launch_leaf_inverse_blocked<T>(LU, ipiv, m, nleaf, Dinv, s);
  const size_t avail = kSmemCap - piv_bytes - (lu_smem ? lu_bytes : 0);
  const int ct_max = (int)std::min<size_t>(avail / ((size_t)m * sizeof(T)), 128);
  const int ntile = ceil_div(m, ct_max), ct = ceil_div(m, ntile);
  const size_t bytes = (size_t)m * ct * sizeof(T) + piv_bytes + (lu_smem ? lu_bytes : 0);
  dim3 grid(ntile, nleaf);
  if (lu_smem) {
    auto k = leaf_inverse_kernel<T, true>;
    cudaError_t e = set_smem(k, bytes);
    if (e != cudaSuccess) return e;
    HODLR_LAUNCH(k, grid, 256, bytes, s, LU, ipiv, m, Dinv, ct);
  } else {
    auto k = leaf_inverse_kernel<T, false>;
    cudaError_t e = set_smem(k, bytes);
    if (e != cudaSuccess) return e;
    HODLR_LAUNCH(k, grid, 256, bytes, s, LU, ipiv, m, Dinv, ct);
  }
  return cudaGetLastError();
}
template cudaError_t launch_leaf_inverse<double>(const double *, const int *, int, int, double *, cudaStream_t);
template cudaError_t launch_leaf_inverse<float>(const float *, const int *, int, int, float *, cudaStream_t);

// ----------------------------------------------------------- leaf apply
// X_i := op(Dinv_i) X_i in place for the rows of every leaf i, columns
// [0, ncols).  One CTA per (leaf, tile of CT = 8192/M columns): the X tile is
// staged whole (so the in-place write is safe), Dinv streams through shared
// memory in 32-column slabs, each thread owns an (M/16) x (CT/16) register
// tile.
template <typename T, int M, bool TRANS>
__global__ void __launch_bounds__(256)
leaf_apply_kernel(const T *__restrict__ Dinv, T *X, long long ldx, int ncols, const int *skip) {
  if (skip && *skip) return;
  constexpr int CT = 8192 / M, KC = 32, RPT = M / 16, CPT = CT / 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sX = reinterpret_cast<T *>(smem_raw);      // M x CT, ld M
  T *sA = sX + M * CT;                          // M x KC slab of op(Dinv), [k][i] layout (ld M)
  const int leaf = blockIdx.y, c0 = blockIdx.x * CT, nc = min(CT, ncols - c0);
  const T *A = Dinv + (long long)leaf * M * M;
  T *Xg = X + (long long)leaf * M + (long long)c0 * ldx;
  const int tid = threadIdx.x, ti = tid & 15, tj = tid >> 4;
  for (int e = tid; e < M * CT; e += 256) {
    const int i = e % M, j = e / M;
    sX[e] = j < nc ? Xg[i + (long long)j * ldx] : T(0);
  }
  T acc[RPT][CPT];
#pragma unroll
  for (int a = 0; a < RPT; ++a)
#pragma unroll
    for (int b = 0; b < CPT; ++b) acc[a][b] = T(0);
  for (int k0 = 0; k0 < M; k0 += KC) {
    __syncthreads();
    // slab: sA[q][i] = op(Dinv)(i, k0 + q)
    for (int e = tid; e < M * KC; e += 256) {
      const int i = e % M, q = e / M;
      sA[q * M + i] = TRANS ? A[(k0 + q) + (long long)i * M] : A[i + (long long)(k0 + q) * M];
    }
    __syncthreads();
#pragma unroll 4
    for (int q = 0; q < KC; ++q) {
      T av[RPT], xv[CPT];
#pragma unroll
      for (int a = 0; a < RPT; ++a) av[a] = sA[q * M + ti + 16 * a];
#pragma unroll
      for (int b = 0; b < CPT; ++b) xv[b] = sX[(k0 + q) + (tj + 16 * b) * M];
#pragma unroll
      for (int a = 0; a < RPT; ++a)
#pragma unroll
        for (int b = 0; b < CPT; ++b) acc[a][b] += av[a] * xv[b];
    }
  }
#pragma unroll
  for (int b = 0; b < CPT; ++b) {
    const int j = tj + 16 * b;
    if (j >= nc) continue;
#pragma unroll
    for (int a = 0; a < RPT; ++a) Xg[ti + 16 * a + (long long)j * ldx] = acc[a][b];
  }
}

// The FP32 leaf-128 case (every mixed-path leaf application but the
// transposed ones) with 8 x 8 register tiles read as float4 runs: 128
// threads per (leaf, 64-column tile); a thread owns rows 4 ti .. 4 ti + 3 and
// 64 + 4 ti .. 64 + 4 ti + 3 and columns 8 tj .. 8 tj + 7.  The X tile is
// staged transposed ([k][column], rows padded to 68 floats) so that both
// operands come as two 16-byte loads: 4 shared loads per 64 FMAs.  The
// result goes back through shared memory for coalesced global stores.
constexpr int kLa128Threads = 128, kLa128CT = 64, kLa128LD = kLa128CT + 4;
constexpr size_t kLa128Smem = (size_t)(128 * kLa128LD + 32 * 128) * sizeof(float);

__device__ __forceinline__ float to_f32(float x) { return x; }
__device__ __forceinline__ float to_f32(double x) { return f64_to_f32_rn(x); }

// The source tile may be another matrix, of FP32 or FP64 (rounded to FP32
// as it is staged): the factorisation's first application reads U in FP64
// and writes Utilde in FP32 with no separate conversion pass.
template <typename S>
__global__ void __launch_bounds__(kLa128Threads, 4)
leaf_apply128_f32_kernel(const float *__restrict__ Dinv, const S *Xs, long long lds, float *X, long long ldx,
                         int ncols, const int *skip) {
  if (skip && *skip) return;
  constexpr int M = 128, CT = kLa128CT, LD = kLa128LD, KC = 32, NT = kLa128Threads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *sXt = reinterpret_cast<float *>(smem_raw);  // [M][LD]: sXt[k * LD + j] = X(k, j)
  float *sA = sXt + M * LD;                           // [KC][M]: sA[q * M + i] = Dinv(i, k0 + q)
  const int leaf = blockIdx.y, c0 = blockIdx.x * CT, nc = min(CT, ncols - c0);
  const float *A = Dinv + (long long)leaf * M * M;
  float *Xg = X + (long long)leaf * M + (long long)c0 * ldx;
  const S *Xsg = Xs + (long long)leaf * M + (long long)c0 * lds;
  const int tid = threadIdx.x, ti = tid & 15, tj = tid >> 4;
  // coalesced along the rows of X; four columns per thread land as one
  // 16-byte store (rows 68 floats apart: a quarter warp covers all banks)
  for (int e = tid; e < M * CT / 4; e += NT) {
    const int i = e % M, j = 4 * (e / M);
    float v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = j + u < nc ? to_f32(Xsg[i + (long long)(j + u) * lds]) : 0.f;
    *reinterpret_cast<float4 *>(sXt + i * LD + j) = make_float4(v[0], v[1], v[2], v[3]);
  }
  // column pairs (8 tj + 2 p, + 1) in packed FP32x2 accumulators: one packed
  // FMA does the two products of a row with an adjacent column pair
  float2 acc[8][4];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int p = 0; p < 4; ++p) acc[a][p] = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < M; k0 += KC) {
    __syncthreads();
    for (int e = tid; e < M * KC / 4; e += NT) {  // the slab, 16-byte copies
      const int i4 = e % (M / 4), q = e / (M / 4);
      reinterpret_cast<float4 *>(sA + q * M)[i4] = reinterpret_cast<const float4 *>(A + (long long)(k0 + q) * M)[i4];
    }
    __syncthreads();
#pragma unroll 2
    for (int q = 0; q < KC; ++q) {
      const float4 a0 = *reinterpret_cast<const float4 *>(sA + q * M + 4 * ti);
      const float4 a1 = *reinterpret_cast<const float4 *>(sA + q * M + 64 + 4 * ti);
      const float4 x0 = *reinterpret_cast<const float4 *>(sXt + (k0 + q) * LD + 8 * tj);
      const float4 x1 = *reinterpret_cast<const float4 *>(sXt + (k0 + q) * LD + 8 * tj + 4);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float2 xp[4] = {make_float2(x0.x, x0.y), make_float2(x0.z, x0.w), make_float2(x1.x, x1.y),
                            make_float2(x1.z, x1.w)};
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int p = 0; p < 4; ++p) acc[a][p] = __ffma2_rn(make_float2(av[a], av[a]), xp[p], acc[a][p]);
    }
  }
  __syncthreads();  // every thread is done with sXt: it takes the result, column-major ld M
  float *sY = sXt;
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    float *col = sY + (8 * tj + b) * M;
    float y[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) y[a] = (b & 1) ? acc[a][b >> 1].y : acc[a][b >> 1].x;
    *reinterpret_cast<float4 *>(col + 4 * ti) = make_float4(y[0], y[1], y[2], y[3]);
    *reinterpret_cast<float4 *>(col + 64 + 4 * ti) = make_float4(y[4], y[5], y[6], y[7]);
  }
  __syncthreads();
  for (int e = tid; e < M * CT; e += NT) {
    const int i = e % M, j = e / M;
    if (j < nc) Xg[i + (long long)j * ldx] = sY[e];
  }
}

template <typename T, int M>
static cudaError_t leaf_apply_m(const T *Dinv, int nleaf, T *X, long long ldx, int ncols, bool trans,
                                const int *skip, cudaStream_t s) {
  constexpr int CT = 8192 / M;
  const size_t bytes = (size_t)M * CT * sizeof(T) + (size_t)M * 32 * sizeof(T);
  dim3 grid(ceil_div(ncols, CT), nleaf);
  if constexpr (std::is_same<T, float>::value && M == 128) {
    if (!trans) {
      auto k = leaf_apply128_f32_kernel<float>;
      cudaError_t e = set_smem(k, kLa128Smem);
      if (e != cudaSuccess) return e;
      HODLR_LAUNCH(k, dim3(ceil_div(ncols, kLa128CT), nleaf), kLa128Threads, kLa128Smem, s, Dinv,
                   (const float *)X, ldx, X, ldx, ncols, skip);
      return cudaGetLastError();
    }
  }
  if (trans) {
    auto k = leaf_apply_kernel<T, M, true>;
    cudaError_t e = set_smem(k, bytes);
    if (e != cudaSuccess) return e;
    HODLR_LAUNCH(k, grid, 256, bytes, s, Dinv, X, ldx, ncols, skip);
  } else {
    auto k = leaf_apply_kernel<T, M, false>;
    cudaError_t e = set_smem(k, bytes);
    if (e != cudaSuccess) return e;
    HODLR_LAUNCH(k, grid, 256, bytes, s, Dinv, X, ldx, ncols, skip);
  }
  return cudaGetLastError();
}

bool leaf_apply_supported(int m) { return m == 64 || m == 128 || m == 256; }

cudaError_t launch_leaf_apply_f64src(const float *Dinv, int m, int nleaf, const double *Xs, long long lds, float *X,
                                     long long ldx, int ncols, DevStatus *st, cudaStream_t s) {
  if (m != 128) return cudaErrorNotSupported;
  if (ncols <= 0 || nleaf <= 0) return cudaSuccess;
  cudaError_t err = cudaSuccess;
  if (leaf_apply_tc_try(Dinv, nleaf, Xs, lds, X, ldx, ncols, st, s, err)) return err;
  auto k = leaf_apply128_f32_kernel<double>;
  cudaError_t e = set_smem(k, kLa128Smem);
  if (e != cudaSuccess) return e;
  HODLR_LAUNCH(k, dim3(ceil_div(ncols, kLa128CT), nleaf), kLa128Threads, kLa128Smem, s, Dinv, Xs, lds, X, ldx, ncols,
               (const int *)nullptr);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_leaf_apply(const T *Dinv, int m, int nleaf, T *X, long long ldx, int ncols, bool trans,
                              const int *skip, cudaStream_t s) {
  if (ncols <= 0 || nleaf <= 0) return cudaSuccess;
  switch (m) {
    case 64: return leaf_apply_m<T, 64>(Dinv, nleaf, X, ldx, ncols, trans, skip, s);
    case 128: return leaf_apply_m<T, 128>(Dinv, nleaf, X, ldx, ncols, trans, skip, s);
    case 256: return leaf_apply_m<T, 256>(Dinv, nleaf, X, ldx, ncols, trans, skip, s);
    default: return cudaErrorInvalidValue;
  }
}
template cudaError_t launch_leaf_apply<double>(const double *, int, int, double *, long long, int, bool,
                                               const int *, cudaStream_t);
template cudaError_t launch_leaf_apply<float>(const float *, int, int, float *, long long, int, bool,
                                              const int *, cudaStream_t);

// ------------------------------------------------------ capacitance factor
// One CTA per node of a depth: S = [I, s.T1u; s.T0u, I] (FP64), LU with
// partial pivoting (stored for inspection), then Sinv = S^{-1} (FP64, and a
// double-word copy when sinv2 is given).
__global__ void __launch_bounds__(256) cap_factor_kernel(CapFactorArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_info;
  const int p = blockIdx.x, node = a.node_base + p;
  const int r = a.r, n2 = 2 * r;
  double *S = reinterpret_cast<double *>(smem_raw);
  double *W = S + n2 * n2;  // n2 x 32 identity tile
  int *piv = reinterpret_cast<int *>(W + n2 * 32);
  const long long o0 = (long long)(2 * p) * a.tb_stride, o1 = (long long)(2 * p + 1) * a.tb_stride;
  auto T = [&](long long off) -> double { return a.Tb32 ? (double)a.Tb32[off] : a.Tb[off]; };
  auto fill_S = [&]() {
    for (int e = threadIdx.x; e < n2 * n2; e += blockDim.x) {
      const int i = e % n2, j = e / n2;
      double v = (i == j) ? 1.0 : 0.0;
      if (i >= r && j < r) v = (a.scale ? a.scale[i - r] : 1.0) * T(o0 + (i - r) + (long long)(a.ucol + j) * r);
      if (i < r && j >= r) v = (a.scale ? a.scale[i] : 1.0) * T(o1 + i + (long long)(a.ucol + j - r) * r);
      S[e] = v;
    }
  };
  fill_S();
  __syncthreads();
  block_getrf<double>(S, n2, n2, piv, &s_info);
  if (s_info && threadIdx.x == 0) report_error(a.st, HODLR_ERR_SINGULAR_CAPACITANCE, node);
  double *gS = a.cap_lu + (long long)node * n2 * n2;
  for (int e = threadIdx.x; e < n2 * n2; e += blockDim.x) gS[e] = S[e];
  for (int e = threadIdx.x; e < n2; e += blockDim.x) a.cap_ipiv[(long long)node * n2 + e] = piv[e];
  // explicit inverse: Gauss-Jordan on a fresh copy of S
  __syncthreads();
  fill_S();
  __syncthreads();
  block_gj_inverse<double>(S, n2, n2, W, piv, &s_info);
  double *gI = a.sinv ? a.sinv + (long long)node * n2 * n2 : nullptr;
  float2 *gI2 = a.sinv2 ? a.sinv2 + (long long)node * n2 * n2 : nullptr;
  float *gI32 = a.sinv32 ? a.sinv32 + (long long)node * n2 * n2 : nullptr;
  for (int e = threadIdx.x; e < n2 * n2; e += blockDim.x) {
    if (gI) gI[e] = S[e];
    if (gI32) gI32[e] = (float)S[e];
    if (gI2) {
      const float h = __double2float_rn(S[e]);
      gI2[e] = make_float2(h, __double2float_rn(S[e] - (double)h));
    }
  }
}

// Same contract with the 2r x 2r system resident in registers (reg_factor.cuh)
// for 2r in {32, 64, 128}.
template <int N2>
__global__ void __launch_bounds__(256, 1) cap_factor_reg_kernel(CapFactorArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_info;
  double *buf = reinterpret_cast<double *>(smem_raw);
  const int p = blockIdx.x, node = a.node_base + p;
  constexpr int r = N2 / 2;
  const long long o0 = (long long)(2 * p) * a.tb_stride, o1 = (long long)(2 * p + 1) * a.tb_stride;
  auto T = [&](long long off) -> double { return a.Tb32 ? (double)a.Tb32[off] : a.Tb[off]; };
  auto load = [&](int i, int j) -> double {
    double v = (i == j) ? 1.0 : 0.0;
    if (i >= r && j < r) v = (a.scale ? a.scale[i - r] : 1.0) * T(o0 + (i - r) + (long long)(a.ucol + j) * r);
    if (i < r && j >= r) v = (a.scale ? a.scale[i] : 1.0) * T(o1 + i + (long long)(a.ucol + j - r) * r);
    return v;
  };
  if (a.sinv32) {
    // mixed path: the LU (and pivots) in FP64, then the inverse the FP32 sweeps
    // apply, by an FP32 Gauss-Jordan sweep on S rounded to FP32
    auto nostore = [](int, int, double) {};
    reg_factor<double, N2>(load, buf, a.cap_lu + (long long)node * N2 * N2, a.cap_ipiv + (long long)node * N2,
                           nostore, false, &s_info);
    if (s_info && threadIdx.x == 0) report_error(a.st, HODLR_ERR_SINGULAR_CAPACITANCE, node);
    __syncthreads();
    float *g32 = a.sinv32 + (long long)node * N2 * N2;
    auto load32 = [&](int i, int j) -> float { return (float)load(i, j); };
    auto store32 = [&](int i, int j, float v) { g32[i + j * N2] = v; };
    int info32 = 0;
    reg_factor<float, N2>(load32, reinterpret_cast<float *>(buf), (float *)nullptr, (int *)nullptr, store32, true,
                          &info32);
    return;
  }
  double *gI = a.sinv + (long long)node * N2 * N2;
  float2 *gI2 = a.sinv2 ? a.sinv2 + (long long)node * N2 * N2 : nullptr;
  auto store = [&](int i, int j, double v) {
    gI[i + j * N2] = v;
    if (gI2) {
      const float h = __double2float_rn(v);
      gI2[i + j * N2] = make_float2(h, __double2float_rn(v - (double)h));
    }
  };
  reg_factor<double, N2>(load, buf, a.cap_lu + (long long)node * N2 * N2, a.cap_ipiv + (long long)node * N2, store,
                         true, &s_info);
  if (s_info && threadIdx.x == 0) report_error(a.st, HODLR_ERR_SINGULAR_CAPACITANCE, node);
}

// Mixed path, 2r <= M (M = 32 or 64; S padded with the identity): one CTA of
// eight warps per node, the system in registers in a column-cyclic layout --
// warp w holds the columns j = w + 8c, lane q the rows q + 32s -- for the
// whole factorisation.  Row interchanges are implicit: rows never move, each
// lane tracks the current position of its rows, so an elimination step
// costs per column one shuffle of the pivot row's entry and the update of
// the rows not yet pivotal; the factors are stored by position at the end.
// Pivot search is warp-local (integer compares of |a|'s bit pattern, ties to
// the lowest position, redux), and each step costs one block barrier: the
// warp owning column k+1 updates, pivots and scales it first and publishes
// its multipliers in a double buffer while the other warps are still on
// step k (lookahead).  The FP64 LU performs dgetf2's operations in its order
// (first row of largest |a|, whole-row interchanges, reciprocal scaling
// unless the pivot is below the safe minimum, rank-1 update of the trailing
// matrix), so factors and pivots equal the explicit-interchange ones bit for
// bit.  The FP32 inverse comes from these factors: the identity rides along
// as FP32 columns in the same layout, receiving the same row operations with
// the rounded multipliers, which leaves L^{-1} P there; an FP32 back
// substitution with U then gives S^{-1} = U^{-1} L^{-1} P.
template <int RS, typename V>
__device__ __forceinline__ V slot_get(const V (&v)[RS], int s) {
  V x = v[0];
#pragma unroll
  for (int q = 1; q < RS; ++q) x = (s == q) ? v[q] : x;
  return x;
}
// Entry of physical row p of a warp-held column (row p at lane p % 32, slot p / 32), to every lane.
template <int RS, typename V>
__device__ __forceinline__ V row_entry(const V (&v)[RS], int p) {
  return __shfl_sync(0xffffffffu, slot_get<RS>(v, p >> 5), p & 31);
}

template <int M, int NW>
__global__ void __launch_bounds__(NW * 32, (NW >= 32 || NW * 32 * (M / NW) >= 4096) ? 1 : (NW >= 16 ? 2 : 3))
cap_factor_cols_kernel(CapFactorArgs a) {
  constexpr int RS = M / 32, CW = M / NW;
  __shared__ double s_l[2][M];   // multipliers by physical row
  __shared__ float s_l32[2][M];
  __shared__ int4 s_piv[2];      // (pivot row, row at position k, pivot row's position, -)
  __shared__ int s_info;
  extern __shared__ float cols_dyn[];
  float *s_u = cols_dyn;         // U rounded to FP32, by position, [j][i] (M * M)
  float *s_z = cols_dyn + M * M; // L^{-1} P by position, [j][i] (M * M)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pn = blockIdx.x, node = a.node_base + pn, r = a.r, n2 = 2 * r;
  const long long o0 = (long long)(2 * pn) * a.tb_stride, o1 = (long long)(2 * pn + 1) * a.tb_stride;
  int *ipiv = a.cap_ipiv + (long long)node * n2;
  double A[CW][RS];
  float Z[CW][RS];
  int pos[RS];  // current position of this lane's rows
#pragma unroll
  for (int s = 0; s < RS; ++s) pos[s] = lane + 32 * s;
#pragma unroll
  for (int c = 0; c < CW; ++c)
#pragma unroll
    for (int s = 0; s < RS; ++s) {
      const int i = lane + 32 * s, j = warp + NW * c;
      double v = (i == j) ? 1.0 : 0.0;
      if (j < n2 && i < n2) {
        auto T = [&](long long off) -> double { return a.Tb32 ? (double)a.Tb32[off] : a.Tb[off]; };
        if (i >= r && j < r) v = (a.scale ? a.scale[i - r] : 1.0) * T(o0 + (i - r) + (long long)(a.ucol + j) * r);
        if (i < r && j >= r) v = (a.scale ? a.scale[i] : 1.0) * T(o1 + i + (long long)(a.ucol + j - r) * r);
      }
      A[c][s] = v;
      Z[c][s] = (i == j) ? 1.f : 0.f;
    }
  if (threadIdx.x == 0) s_info = 0;

  // Owner warp of column k (register column c), rows at positions >= k
  // still unpivoted: pivot choice, scaling, publication in buffer k & 1.
  auto pivot_column = [&](int k, double(&col)[RS]) {
    unsigned long long best = 0;
    int bpos = M;
#pragma unroll
    for (int s = 0; s < RS; ++s) {
      unsigned long long key = static_cast<unsigned long long>(__double_as_longlong(col[s])) & 0x7fffffffffffffffull;
      if (key > 0x7ff0000000000000ull) key = 0;  // NaN is never preferred
      if (pos[s] >= k && pos[s] < n2 && (bpos == M || key > best || (key == best && pos[s] < bpos))) {
        best = key;
        bpos = pos[s];
      }
    }
    const unsigned hi = static_cast<unsigned>(best >> 32), lo = static_cast<unsigned>(best);
    const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
    const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
    const int pp = static_cast<int>(
        __reduce_min_sync(0xffffffffu, (hi == mhi && lo == mlo) ? static_cast<unsigned>(bpos) : static_cast<unsigned>(M)));
    int pb = 0, pa = 0;  // physical rows at positions pp and k
#pragma unroll
    for (int s = 0; s < RS; ++s) {
      const unsigned mb = __ballot_sync(0xffffffffu, pos[s] == pp), ma = __ballot_sync(0xffffffffu, pos[s] == k);
      if (mb) pb = 32 * s + __ffs(mb) - 1;
      if (ma) pa = 32 * s + __ffs(ma) - 1;
    }
    const double pv = row_entry<RS>(col, pb);
    const unsigned long long pbits = static_cast<unsigned long long>(__double_as_longlong(pv)) & 0x7fffffffffffffffull;
    const bool zero = pbits == 0, tiny = pbits < 0x0010000000000000ull;  // |pv| < DBL_MIN
    const double rcp = zero ? 0.0 : 1.0 / pv;
    const int b = k & 1;
#pragma unroll
    for (int s = 0; s < RS; ++s) {
      const int phys = lane + 32 * s;
      const int np = phys == pb ? k : (phys == pa ? pp : pos[s]);  // position after the interchange
      double l = 0.0;
      if (np > k && np < n2) {
        l = col[s];
        if (!zero) l = tiny ? l / pv : l * rcp;
        col[s] = l;
      }
      s_l[b][phys] = l;
      s_l32[b][phys] = static_cast<float>(l);
    }
    if (lane == 0) {
      s_piv[b] = make_int4(pb, pa, pp, 0);
      ipiv[k] = pp + 1;
      if (zero && s_info == 0) s_info = k + 1;
    }
  };

  if (warp == 0) pivot_column(0, A[0]);
  __syncthreads();
  for (int k = 0; k < n2; ++k) {
    const int b = k & 1;
    const int4 pv4 = s_piv[b];
    const int pb = pv4.x, pa = pv4.y, pp = pv4.z;
    bool rem[RS];
    double l[RS];
    float l32[RS];
#pragma unroll
    for (int s = 0; s < RS; ++s) {
      const int phys = lane + 32 * s;
      pos[s] = phys == pb ? k : (phys == pa ? pp : pos[s]);
      rem[s] = pos[s] > k && pos[s] < n2;
      l[s] = s_l[b][phys];
      l32[s] = s_l32[b][phys];
    }
    auto update = [&](double(&v)[RS]) {
      const double u = row_entry<RS>(v, pb);
#pragma unroll
      for (int s = 0; s < RS; ++s)
        if (rem[s]) v[s] -= l[s] * u;
    };
    // lookahead: the owner of column k+1 finishes it and publishes step k+1
    const int k1 = k + 1;
    if (k1 < n2 && (k1 % NW) == warp) {
#pragma unroll
      for (int c = 0; c < CW; ++c)  // constant register index: the column stays in registers
        if (warp + NW * c == k1) {
          update(A[c]);
          pivot_column(k1, A[c]);
        }
    }
#pragma unroll
    for (int c = 0; c < CW; ++c) {
      const int j = warp + NW * c;
      if (j < n2 && j > k1) update(A[c]);
      if (j < n2) {  // identity column j: the same row operation with the FP32 multipliers
        const float z = row_entry<RS>(Z[c], pb);
#pragma unroll
        for (int s = 0; s < RS; ++s)
          if (rem[s]) Z[c][s] -= l32[s] * z;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && s_info) report_error(a.st, HODLR_ERR_SINGULAR_CAPACITANCE, node);
  double *gS = a.cap_lu + (long long)node * n2 * n2;
#pragma unroll
  for (int c = 0; c < CW; ++c)
#pragma unroll
    for (int s = 0; s < RS; ++s) {
      const int j = warp + NW * c;
      s_u[pos[s] + j * M] = static_cast<float>(A[c][s]);
      s_z[pos[s] + j * M] = Z[c][s];
      if (pos[s] < n2 && j < n2) gS[pos[s] + (long long)j * n2] = A[c][s];
    }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < CW; ++c)
#pragma unroll
    for (int s = 0; s < RS; ++s) Z[c][s] = s_z[lane + 32 * s + (warp + NW * c) * M];
  // X = U^{-1} Z, column by column in the warps that hold them (rows by position now)
  for (int k = n2 - 1; k >= 0; --k) {
    const float rd = 1.f / s_u[k + k * M];
    float u[RS];
#pragma unroll
    for (int s = 0; s < RS; ++s) u[s] = s_u[lane + 32 * s + k * M];
#pragma unroll
    for (int c = 0; c < CW; ++c) {
      if (warp + NW * c >= n2) continue;
      const float x = row_entry<RS>(Z[c], k) * rd;
#pragma unroll
      for (int s = 0; s < RS; ++s) {
        const int i = lane + 32 * s;
        if (i == k) Z[c][s] = x;
        else if (i < k) Z[c][s] -= u[s] * x;
      }
    }
  }
  float *g32 = a.sinv32 + (long long)node * n2 * n2;
#pragma unroll
  for (int c = 0; c < CW; ++c)
#pragma unroll
    for (int s = 0; s < RS; ++s) {
      const int i = lane + 32 * s, j = warp + NW * c;
      if (i < n2 && j < n2) g32[i + (long long)j * n2] = Z[c][s];
    }
}

template <int M, int NW>
static cudaError_t launch_cap_cols(const CapFactorArgs &a, cudaStream_t s) {
  const size_t bytes = (size_t)2 * M * M * sizeof(float);
  cudaError_t e = set_smem(cap_factor_cols_kernel<M, NW>, bytes);
  if (e != cudaSuccess) return e;
  HODLR_LAUNCH((cap_factor_cols_kernel<M, NW>), a.nnode, NW * 32, bytes, s, a);
  return cudaGetLastError();
}

template <int N2>
static cudaError_t launch_cap_reg(const CapFactorArgs &a, cudaStream_t s) {
  const size_t bytes = (size_t)N2 * N2 * 8;
  auto k = cap_factor_reg_kernel<N2>;
  cudaError_t e = set_smem(k, bytes);
  if (e != cudaSuccess) return e;
  HODLR_LAUNCH(k, a.nnode, 256, bytes, s, a);
  return cudaGetLastError();
}

cudaError_t launch_cap_factor(const CapFactorArgs &a, cudaStream_t s) {
  if (a.nnode <= 0) return cudaSuccess;
  if (a.r < 1 || a.r > 64) return cudaErrorInvalidValue;
  const int n2 = 2 * a.r;
  if (a.sinv32 && n2 <= 32) return launch_cap_cols<32, 8>(a, s);
  if (a.sinv32 && n2 <= 64) {
    // warps per system: the tuned value, or by level -- a level with at most one
    // system per SM runs each pivot chain with 32 warps (one CTA per SM), up to
    // two per SM with 16, the wide levels keep three 8-warp systems per SM
    int w = current_tuning().cap_warps;
    if (w == 0) w = a.nnode <= kNumSMs ? 32 : (a.nnode <= 2 * kNumSMs ? 16 : 8);
    if (w == 32) return launch_cap_cols<64, 32>(a, s);
    if (w == 16) return launch_cap_cols<64, 16>(a, s);
    return launch_cap_cols<64, 8>(a, s);
  }
  if (a.sinv32) return launch_cap_cols<128, 16>(a, s);
  if (n2 == 32) return launch_cap_reg<32>(a, s);
  if (n2 == 64) return launch_cap_reg<64>(a, s);
  if (n2 == 128) return launch_cap_reg<128>(a, s);
  const size_t bytes = (size_t)n2 * n2 * 8 + (size_t)n2 * 32 * 8 + (size_t)n2 * 4 + 16;
  cudaError_t e = set_smem(cap_factor_kernel, bytes);
  if (e != cudaSuccess) return e;
  HODLR_LAUNCH(cap_factor_kernel, a.nnode, 256, bytes, s, a);
  return cudaGetLastError();
}

// ------------------------------------------------------- capacitance apply
// eta_p = op(Sinv_p) RHS_p for the nodes of one depth, RHS_p built from the
// children's T blocks: forward [s.T1; s.T0] with Sinv, transposed [T0; T1]
// with Sinv^T.  FP64 (DFMA) or double-word (FP32 pipes, FP64-accurate).
// grid (column tiles of 32, nnode); each thread owns MT x 4 outputs.
__device__ __forceinline__ void dw2_fma(float ah, float al, float xh, float xl, float &sh, float &sl) {
  const float pr = ah * xh;
  const float e = fmaf(ah, xh, -pr);
  const float s = sh + pr;
  const float bb = s - sh;
  const float t = (sh - (s - bb)) + (pr - bb);
  sh = s;
  sl += t + e;
  sl = fmaf(ah, xl, sl);
  sl = fmaf(al, xh, sl);
}

template <int MT, bool DW>
__global__ void __launch_bounds__(256) cap_apply_kernel(CapApplyArgs a) {
  if (a.skip && *a.skip) return;
  using E = typename std::conditional<DW, float2, double>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int r = a.r, n2 = 2 * r;
  constexpr int NP = MT * 32;  // padded rows
  E *sS = reinterpret_cast<E *>(smem_raw);   // [q][i], NP x NP (op(Sinv)(i, q) at sS[q*NP + i])
  E *sR = sS + NP * NP;                      // [q][j], NP x 32
  const int p = blockIdx.y;
  const int node = a.node_base + p;
  const double *Sg = a.sinv + (long long)node * n2 * n2;
  const float2 *Sg2 = a.sinv2 ? a.sinv2 + (long long)node * n2 * n2 : nullptr;
  // op(Sinv) is staged once per CTA; the CTA then walks its column tiles
  // (blockIdx.x, + gridDim.x, ...)
  for (int e = threadIdx.x; e < NP * NP; e += blockDim.x) {
    const int i = e % NP, q = e / NP;
    E v;
    if constexpr (DW) {
      v = make_float2(0.f, 0.f);
      if (i < n2 && q < n2) v = a.trans ? Sg2[q + (long long)i * n2] : Sg2[i + (long long)q * n2];
    } else {
      v = 0.0;
      if (i < n2 && q < n2) v = a.trans ? Sg[q + (long long)i * n2] : Sg[i + (long long)q * n2];
    }
    sS[q * NP + i] = v;
  }
  const double *T0 = a.Tb + (long long)(2 * p) * a.tb_stride;
  const double *T1 = a.Tb + (long long)(2 * p + 1) * a.tb_stride;
  for (int c0 = blockIdx.x * 32; c0 < a.C; c0 += gridDim.x * 32) {
  const int nc = min(32, a.C - c0);
  __syncthreads();  // the previous tile's reads of sR are done
  for (int e = threadIdx.x; e < NP * 32; e += blockDim.x) {
    const int q = e % NP, j = e / NP;
    double v = 0.0;
    if (q < n2 && j < nc) {
      if (!a.trans)
        v = (q < r) ? (a.scale ? a.scale[q] : 1.0) * T1[q + (long long)(c0 + j) * r]
                    : (a.scale ? a.scale[q - r] : 1.0) * T0[(q - r) + (long long)(c0 + j) * r];
      else
        v = (q < r) ? T0[q + (long long)(c0 + j) * r] : T1[(q - r) + (long long)(c0 + j) * r];
    }
    if constexpr (DW) {
      const float h = __double2float_rn(v);
      sR[j * NP + q] = make_float2(h, __double2float_rn(v - (double)h));
    } else {
      sR[j * NP + q] = v;
    }
  }
  __syncthreads();
  const int ti = threadIdx.x & 31, tj = threadIdx.x >> 5;
  double *eta = a.eta + (long long)p * n2 * a.C;
  if constexpr (DW) {
    float sh[MT][4], sl[MT][4];
#pragma unroll
    for (int u = 0; u < MT; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) sh[u][v] = sl[u][v] = 0.f;
    for (int q = 0; q < n2; ++q) {
      float2 sv[MT];
#pragma unroll
      for (int u = 0; u < MT; ++u) sv[u] = sS[q * NP + ti + 32 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float2 rv = sR[(tj + 8 * v) * NP + q];
#pragma unroll
        for (int u = 0; u < MT; ++u) dw2_fma(sv[u].x, sv[u].y, rv.x, rv.y, sh[u][v], sl[u][v]);
      }
      if ((q & 31) == 31) {
#pragma unroll
        for (int u = 0; u < MT; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const float s = sh[u][v] + sl[u][v];
            sl[u][v] = sl[u][v] - (s - sh[u][v]);
            sh[u][v] = s;
          }
      }
    }
#pragma unroll
    for (int u = 0; u < MT; ++u) {
      const int i = ti + 32 * u;
      if (i >= n2) continue;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int j = tj + 8 * v;
        if (j >= nc) continue;
        const double val = (double)sh[u][v] + (double)sl[u][v];
        if (a.eta32)
          a.eta32[(long long)p * n2 * a.C + i + (long long)(c0 + j) * n2] =
              (float)(a.out_scale ? val * a.out_scale[i % r] : val);
        else
          eta[i + (long long)(c0 + j) * n2] = val;
      }
    }
  } else {
    double acc[MT][4];
#pragma unroll
    for (int u = 0; u < MT; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
    for (int q = 0; q < n2; ++q) {
      double sv[MT];
#pragma unroll
      for (int u = 0; u < MT; ++u) sv[u] = sS[q * NP + ti + 32 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double rv = sR[(tj + 8 * v) * NP + q];
#pragma unroll
        for (int u = 0; u < MT; ++u) acc[u][v] = fma(sv[u], rv, acc[u][v]);
      }
    }
#pragma unroll
    for (int u = 0; u < MT; ++u) {
      const int i = ti + 32 * u;
      if (i >= n2) continue;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int j = tj + 8 * v;
        if (j >= nc) continue;
        if (a.eta32)
          a.eta32[(long long)p * n2 * a.C + i + (long long)(c0 + j) * n2] =
              (float)(a.out_scale ? acc[u][v] * a.out_scale[i % r] : acc[u][v]);
        else
          eta[i + (long long)(c0 + j) * n2] = acc[u][v];
      }
    }
  }
  }  // column tiles
}

// Mixed path: eta = op(Sinv) RHS in FP32 (the FP32 inverse against the FP32
// T blocks), written as FP32 for the FP32 updates (eta32, rows scaled by
// out_scale).  Same tiling as above.
template <int NP, int CPT>
__global__ void __launch_bounds__(256) cap_apply_f32_kernel(CapApplyArgs a) {
  // eta = op(S^-1) RHS for one node and CT columns at a time: thread (rg, ct)
  // owns rows 4 rg .. 4 rg + 3 and the column quads 4 ct + 4 CTH g (g < CPT / 4);
  // the inverse ([q][i]) and the right-hand sides ([q][j]) are read as float4
  // runs, every output summed over q in increasing order
  constexpr int RG = NP / 4, CTH = 256 / RG, CT = CTH * CPT, SP = NP + 4, RP = CT + 4, NG = CPT / 4;
  if (a.skip && *a.skip) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int r = a.r, n2 = 2 * r;
  float *sS = reinterpret_cast<float *>(smem_raw);  // [q][i], row stride SP
  float *sR = sS + NP * SP;                          // [q][j], row stride RP
  const int p = blockIdx.y;
  const int node = a.node_base + p;
  const float *Sg = a.sinv32 + (long long)node * n2 * n2;
  for (int e = threadIdx.x; e < NP * NP; e += blockDim.x) {
    const int i = e % NP, q = e / NP;
    float v = 0.f;
    if (i < n2 && q < n2) v = a.trans ? Sg[q + (long long)i * n2] : Sg[i + (long long)q * n2];
    sS[q * SP + i] = v;
  }
  const float *T0 = a.Tb32 + (long long)(2 * p) * a.tb_stride;
  const float *T1 = a.Tb32 + (long long)(2 * p + 1) * a.tb_stride;
  const int rg = threadIdx.x % RG, ct = threadIdx.x / RG;
  const bool vec_out = (n2 & 3) == 0;
  float *E = a.eta32 + (long long)p * n2 * a.C;
  for (int c0 = blockIdx.x * CT; c0 < a.C; c0 += gridDim.x * CT) {
    const int nc = min(CT, a.C - c0);
    __syncthreads();
    // four columns per task: loads coalesced over q, one float4 store per task
    // (consecutive q land on distinct bank quads: RP / 4 is odd)
    for (int e = threadIdx.x; e < NP * (CT / 4); e += blockDim.x) {
      const int q = e % NP, j4 = 4 * (e / NP);
      const float *src = nullptr;
      float scv = 1.f;
      if (q < n2) {
        if (!a.trans) {
          src = q < r ? T1 + q : T0 + (q - r);
          if (a.scale) scv = (float)a.scale[q < r ? q : q - r];
        } else {
          src = q < r ? T0 + q : T1 + (q - r);
        }
      }
      float v[4];
#pragma unroll
      for (int w = 0; w < 4; ++w) v[w] = (src && j4 + w < nc) ? scv * src[(long long)(c0 + j4 + w) * r] : 0.f;
      *reinterpret_cast<float4 *>(sR + q * RP + j4) = make_float4(v[0], v[1], v[2], v[3]);
    }
    __syncthreads();
    float acc[4][CPT];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < CPT; ++v) acc[u][v] = 0.f;
    for (int q = 0; q < n2; ++q) {
      const float4 sv = *reinterpret_cast<const float4 *>(sS + q * SP + 4 * rg);
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const float4 rv = *reinterpret_cast<const float4 *>(sR + q * RP + 4 * ct + 4 * CTH * g);
        const float su[4] = {sv.x, sv.y, sv.z, sv.w}, rw[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int w = 0; w < 4; ++w) acc[u][4 * g + w] = fmaf(su[u], rw[w], acc[u][4 * g + w]);
      }
    }
    float sc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = 4 * rg + u;
      sc[u] = (i < n2 && a.out_scale) ? (float)a.out_scale[i % r] : 1.f;
    }
#pragma unroll
    for (int g = 0; g < NG; ++g)
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const int j = 4 * ct + 4 * CTH * g + w;
        if (j >= nc || 4 * rg >= n2) continue;
        float *o = E + 4 * rg + (long long)(c0 + j) * n2;
        if (vec_out) {
          *reinterpret_cast<float4 *>(o) =
              make_float4(acc[0][4 * g + w] * sc[0], acc[1][4 * g + w] * sc[1], acc[2][4 * g + w] * sc[2],
                          acc[3][4 * g + w] * sc[3]);
        } else {
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (4 * rg + u < n2) o[u] = acc[u][4 * g + w] * sc[u];
        }
      }
  }
}

cudaError_t launch_cap_apply(const CapApplyArgs &a, cudaStream_t s) {
  if (a.Tb32 && a.sinv32 && a.eta32) {
    if (a.nnode <= 0 || a.C <= 0) return cudaSuccess;
    if (a.r < 1 || a.r > 64) return cudaErrorInvalidValue;
    const int n2 = 2 * a.r;
    // NP rows (n2 padded), CPT columns per thread: CT = (256 / (NP / 4)) * CPT columns per pass
#define HODLR_CAPF(NPV, CPTV)                                                                        \
  {                                                                                                  \
    constexpr int CT = (256 / (NPV / 4)) * CPTV;                                                     \
    const size_t bytes = sizeof(float) * ((size_t)NPV * (NPV + 4) + (size_t)NPV * (CT + 4));         \
    const int tiles = ceil_div(a.C, CT);                                                             \
    const int groups = std::max(1, std::min(tiles, ceil_div(4 * kNumSMs, a.nnode)));                 \
    auto k = cap_apply_f32_kernel<NPV, CPTV>;                                                        \
    cudaError_t e = set_smem(k, bytes);                                                              \
    if (e != cudaSuccess) return e;                                                                  \
    HODLR_LAUNCH(k, dim3(groups, a.nnode), 256, bytes, s, a);                                        \
  }
    if (n2 <= 32) HODLR_CAPF(32, 4)
    else if (n2 <= 64) { if (a.C <= 64) HODLR_CAPF(64, 4) else HODLR_CAPF(64, 8) }
    else { if (a.C <= 32) HODLR_CAPF(128, 4) else HODLR_CAPF(128, 8) }
#undef HODLR_CAPF
    return cudaGetLastError();
  }
  if (a.nnode <= 0 || a.C <= 0) return cudaSuccess;
  if (a.r < 1 || a.r > 64) return cudaErrorInvalidValue;
  const int n2 = 2 * a.r;
  const int MT = n2 <= 32 ? 1 : (n2 <= 64 ? 2 : 4);
  const int NP = MT * 32;
  const bool dw = a.sinv2 != nullptr;
  const size_t es = dw ? sizeof(float2) : sizeof(double);
  const size_t bytes = (size_t)NP * NP * es + (size_t)NP * 32 * es;
  // enough CTAs to fill the GPU, each covering several column tiles of its node
  const int tiles = ceil_div(a.C, 32);
  const int groups = std::max(1, std::min(tiles, ceil_div(4 * 152, a.nnode)));
  dim3 grid(groups, a.nnode);
#define HODLR_CAPA(MTV, DWV)                                   \
  {                                                            \
    auto k = cap_apply_kernel<MTV, DWV>;                       \
    cudaError_t e = set_smem(k, bytes);                        \
    if (e != cudaSuccess) return e;                            \
    HODLR_LAUNCH(k, grid, 256, bytes, s, a);                   \
  }
  if (dw) {
    if (MT == 1) HODLR_CAPA(1, true) else if (MT == 2) HODLR_CAPA(2, true) else HODLR_CAPA(4, true)
  } else {
    if (MT == 1) HODLR_CAPA(1, false) else if (MT == 2) HODLR_CAPA(2, false) else HODLR_CAPA(4, false)
  }
#undef HODLR_CAPA
  return cudaGetLastError();
}

}  // namespace hodlr
