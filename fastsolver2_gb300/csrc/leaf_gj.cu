// K1' (mixed path, leaf 128): the explicit FP32 inverse of every leaf block,
// one CTA per leaf, by a blocked Gauss-Jordan elimination with implicit row
// pivoting.
//
// Replaces, for the mixed-precision factorisation, the leaf dgesv of
// fastSolver2's hsolve (src/tasks/leaf_solve.cc:80-92): the sweeps apply the
// leaf inverse as a GEMM, so the factorisation only needs A^{-1}; the LU
// factors themselves (an output of the library, not an input of any sweep)
// are formed on request by the LU kernel.
//
// Layout.  Warp w of the 16 warps owns columns [8 w, 8 w + 8) of the block
// ("slab" w) for all 128 rows, lane l rows l, l + 32, l + 64, l + 96: 32
// registers per thread, the whole block in registers.
//
// Algorithm (in-place Gauss-Jordan; rows are never moved).  Step k picks the
// pivot p_k among the rows not yet used as pivots: a row of maximal |a| in
// column k, the first one in storage order among those whose |a| agree in
// their leading 17 significant bits (IDAMAX's rule up to that truncation,
// netlib_blas/idamax.f:52); a zero or subnormal maximum is a zero pivot
// (HODLR_ERR_SINGULAR_LEAF).  With pv = a[p_k][k], the pivot row becomes
// a[p_k][:] / pv with 1 / pv in column k, and every other row i gets
// a[i][:] -= a[i][k] * (new pivot row), with -a[i][k] / pv in column k.
// Afterwards column j holds column p_j of the accumulated transform E
// (E A = the permutation with ones at (p_k, k)), so
// A^{-1}[k][p_j] = M[p_k][j]: the output is scattered with both
// permutations.
//
// Blocking.  Block b = the 8 steps on slab b.  Warp b runs them on its own
// registers, warp-synchronously: the pivot search is one redux.sync.max over
// keys (|a| bits, row), the pivot row is broadcast by shuffles, and the
// pivot row's own update is folded into the FMAs of all rows (scale 0 and
// multiplier -1 give exactly the scaled pivot row).
// The panel then holds W, the block's transform restricted to its columns.
// For every other column x the 8 steps amount to x_new = (x with the pivot
// rows zeroed) + W * x[p_8b .. p_8b+7]: each other warp gathers its slab's 8
// pivot rows and applies that rank-8 update with packed FMAs.  One block
// barrier per block: warp b + 1 starts its panel as soon as its own update
// of block b is done, so a panel overlaps the other warps' updates.
#include "kernels.cuh"

namespace hodlr {

namespace {
constexpr int kGjM = 128, kGjSW = 8, kGjWarps = kGjM / kGjSW, kGjRPL = kGjM / 32;
constexpr unsigned kGjMag = 0x7FFFFF80u;  // |a| bits kept in a pivot key (the low 7 carry the row)

// FP64 -> FP32 with round-to-nearest-even, from the IEEE 754 bit patterns on
// the integer pipes (GB300's FP64 pipe, which F2F.F32.F64 uses, runs at 1/64
// of the FP32 rate).  Results that would be subnormal, zero, overflow, or
// inputs that are not finite take the hardware conversion.  *finite gets
// whether x is finite.
__device__ __forceinline__ float gj_f64_to_f32(double x, bool *finite) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  const int e = (int)((hi >> 20) & 0x7FFu);
  *finite = e != 0x7FF;
  if (e < 1023 - 126 || e > 1023 + 127) return __double2float_rn(x);
  // mantissa bits 51..29 kept, 28..0 rounded off (half = bit 28)
  const unsigned m23 = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  const unsigned rest = lo & 0x1FFFFFFFu, half = 0x10000000u;
  unsigned bits = ((unsigned)(e - 1023 + 127) << 23) + m23;
  bits += (rest > half || (rest == half && (m23 & 1u))) ? 1u : 0u;  // a carry rounds into the exponent
  return __uint_as_float((hi & 0x80000000u) | bits);
}

// 1 / x to within one unit in the last place (MUFU reciprocal); x normal.
__device__ __forceinline__ float gj_rcp(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

struct GjShared {
  float W[2][kGjSW][kGjM];          // the block's panel, [k][row] (double buffer by block parity)
  float R[kGjWarps][kGjSW][kGjSW];  // per warp: its slab's pivot rows [k][j]
  int pall[kGjM];                   // pivot row of step k
  signed char pos[2][kGjM];         // per block parity: step in the block of each pivot row, else -1
  unsigned char qstep[kGjM];        // step at which each row was the pivot
  int info;                         // first zero pivot (step + 1), else 0
};
}  // namespace

__global__ void __launch_bounds__(512, 2)
leaf_gj_inverse_kernel(const double *__restrict__ D, long long d_ld, long long d_stride, DevStatus *st,
                       float *__restrict__ Dinv) {
  __shared__ __align__(16) GjShared sm;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double *Dg = D + (long long)blockIdx.x * d_stride;

  // this warp's slab: a[q][j] = A[lane + 32 q][8 warp + j]
  float a[kGjRPL][kGjSW];
  bool bad = false;
#pragma unroll
  for (int j = 0; j < kGjSW; ++j)
#pragma unroll
    for (int q = 0; q < kGjRPL; ++q) {
      bool fin;
      a[q][j] = gj_f64_to_f32(Dg[(lane + 32 * q) + (long long)(kGjSW * warp + j) * d_ld], &fin);
      bad |= !fin;
    }
  for (int e = threadIdx.x; e < 2 * kGjM; e += blockDim.x) (&sm.pos[0][0])[e] = -1;
  if (threadIdx.x == 0) sm.info = 0;
  if (__syncthreads_or(bad)) {
    if (threadIdx.x == 0) report_error(st, HODLR_ERR_NONFINITE_INPUT, (long long)blockIdx.x * kGjM);
    return;
  }

  unsigned used = 0;  // bit q: row lane + 32 q is already a pivot (kept by every lane for its rows)
  for (int b = 0; b < kGjWarps; ++b) {
    const int par = b & 1;
    if (warp == b) {
      // -------------------------------------------------------------- panel
      if (b >= 2 && lane < kGjSW) sm.pos[par][sm.pall[(b - 2) * kGjSW + lane]] = -1;  // block b-2's marks
      int zero_step = 0;
#pragma unroll
      for (int c = 0; c < kGjSW; ++c) {
        unsigned key = 0;  // used rows key 0: every unused row's key is larger, or row 127's is 0 too
#pragma unroll
        for (int q = 0; q < kGjRPL; ++q)
          if (!((used >> q) & 1u))
            key = max(key, (__float_as_uint(a[q][c]) & kGjMag) | (unsigned)(127 - lane - 32 * q));
        const unsigned kmax = __reduce_max_sync(0xffffffffu, key);
        const int p = 127 - (int)(kmax & 127u);
        const int owner = p & 31, qq = p >> 5;
        const bool zero = (kmax & 0x7F800000u) == 0;  // zero or subnormal: no usable pivot
        if (zero && zero_step == 0) zero_step = kGjSW * b + c + 1;
        if (lane == owner) used |= 1u << qq;
        if (lane == 0) {
          sm.pall[kGjSW * b + c] = p;
          sm.pos[par][p] = (signed char)c;
          sm.qstep[p] = (unsigned char)(kGjSW * b + c);
        }
        float rp[kGjSW];  // the pivot row, by shuffles from its owner (qq is uniform across the warp)
        switch (qq) {
#define HODLR_GJ_ROW(Q)                                                                                   \
  case Q:                                                                                                 \
    _Pragma("unroll") for (int j = 0; j < kGjSW; ++j) rp[j] = __shfl_sync(0xffffffffu, a[Q][j], owner);  \
    break;
          HODLR_GJ_ROW(0) HODLR_GJ_ROW(1) HODLR_GJ_ROW(2) HODLR_GJ_ROW(3)
#undef HODLR_GJ_ROW
        }
        const float inv = zero ? 0.0f : gj_rcp(rp[c]);
        float rn[kGjSW];
#pragma unroll
        for (int j = 0; j < kGjSW; ++j) rn[j] = (j == c) ? inv : rp[j] * inv;
        // every row i: a[i][j] <- s_i a[i][j] - l_i rn[j] (column c: 0 - l_i rn[c]); other rows
        // s = 1, l = a[i][c]; the pivot row s = 0, l = -1 (it becomes rn exactly)
#pragma unroll
        for (int q = 0; q < kGjRPL; ++q) {
          const bool isp = lane == owner && q == qq;
          const float sq = isp ? 0.0f : 1.0f, nl = isp ? 1.0f : -a[q][c];
#pragma unroll
          for (int j = 0; j < kGjSW; j += 2) {
            const float2 sc = make_float2(j == c ? 0.0f : sq, j + 1 == c ? 0.0f : sq);
            float2 x = __fmul2_rn(make_float2(a[q][j], a[q][j + 1]), sc);
            x = __ffma2_rn(make_float2(nl, nl), make_float2(rn[j], rn[j + 1]), x);
            a[q][j] = x.x;
            a[q][j + 1] = x.y;
          }
        }
      }
      // the panel W, [k][row]
#pragma unroll
      for (int k = 0; k < kGjSW; ++k)
#pragma unroll
        for (int q = 0; q < kGjRPL; ++q) sm.W[par][k][lane + 32 * q] = a[q][k];
      if (lane == 0 && zero_step && sm.info == 0) sm.info = zero_step;
    }
    __syncthreads();  // panel b ready; every update of block b-1 done
    if (warp != b) {
      // ------------------------------------------------------- rank-8 update
      float(*R)[kGjSW] = sm.R[warp];
#pragma unroll
      for (int q = 0; q < kGjRPL; ++q) {
        const int kq = sm.pos[par][lane + 32 * q];
        if (kq >= 0) {  // one of the block's pivot rows: gather it; its new value is W's row alone
          reinterpret_cast<float4 *>(R[kq])[0] = make_float4(a[q][0], a[q][1], a[q][2], a[q][3]);
          reinterpret_cast<float4 *>(R[kq])[1] = make_float4(a[q][4], a[q][5], a[q][6], a[q][7]);
          used |= 1u << q;
        }
        const float keep = kq >= 0 ? 0.0f : 1.0f;
#pragma unroll
        for (int j = 0; j < kGjSW; j += 2) {
          const float2 x = __fmul2_rn(make_float2(a[q][j], a[q][j + 1]), make_float2(keep, keep));
          a[q][j] = x.x;
          a[q][j + 1] = x.y;
        }
      }
      __syncwarp();
#pragma unroll
      for (int k = 0; k < kGjSW; ++k) {
        const float4 r0 = reinterpret_cast<const float4 *>(R[k])[0];
        const float4 r1 = reinterpret_cast<const float4 *>(R[k])[1];
        const float rk[kGjSW] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
#pragma unroll
        for (int q = 0; q < kGjRPL; ++q) {
          const float w = sm.W[par][k][lane + 32 * q];
#pragma unroll
          for (int j = 0; j < kGjSW; j += 2) {
            const float2 x = __ffma2_rn(make_float2(w, w), make_float2(rk[j], rk[j + 1]),
                                        make_float2(a[q][j], a[q][j + 1]));
            a[q][j] = x.x;
            a[q][j + 1] = x.y;
          }
        }
      }
      __syncwarp();  // R is rewritten by the next block's gather
    }
  }
  __syncthreads();  // every pivot recorded
  if (threadIdx.x == 0 && sm.info) report_error(st, HODLR_ERR_SINGULAR_LEAF, blockIdx.x);
  // A^{-1}[qstep[r]][p_j] = M[r][j]
  float *out = Dinv + (long long)blockIdx.x * kGjM * kGjM;
#pragma unroll
  for (int j = 0; j < kGjSW; ++j) {
    const int pj = sm.pall[kGjSW * warp + j];
#pragma unroll
    for (int q = 0; q < kGjRPL; ++q) out[sm.qstep[lane + 32 * q] + pj * kGjM] = a[q][j];
  }
}

cudaError_t launch_leaf_gj_inverse_f32(const double *D, long long d_ld, long long d_stride, int m, int nleaf,
                                       DevStatus *st, float *Dinv, cudaStream_t s) {
  if (m != kGjM) return cudaErrorInvalidValue;
  if (nleaf <= 0) return cudaSuccess;
  HODLR_LAUNCH(leaf_gj_inverse_kernel, nleaf, 512, 0, s, D, d_ld, d_stride, st, Dinv);
  return cudaGetLastError();
}

}  // namespace hodlr
