// Tensor-core residual products by exact slicing (see ozaki.cuh): the digit
// kernels and three bf16 mma.sync GEMMs -- leaf term, level reductions
// V^T X, level updates U T' -- with the double-word combination of the
// exact per-diagonal FP32 sums in their epilogues.
//
// MMA: mma.sync.m16n8k16 bf16 x bf16 -> f32.  Fragments (lane = 4 g + t):
// A (16 x 16, row-major) a0 = (g, 2t..2t+1), a1 = (g+8, 2t..), a2 = (g,
// 8+2t..), a3 = (g+8, 8+2t..); B (16 x 8, k contiguous per column) b0 =
// (2t..2t+1, g), b1 = (8+2t.., g); C c0,c1 = (g, 2t..2t+1), c2,c3 = (g+8, ..).
// Shared-memory tiles keep k contiguous with rows padded by 8 bf16 (row
// stride 4 words mod 32), so the eight rows of a fragment load hit distinct
// banks.
#include <algorithm>

#include "kernels.cuh"
#include "ozaki.cuh"
#include "tma.cuh"

namespace hodlr {

// ------------------------------------------------------------------ digits
// All on the integer pipes (GB300 issues FP64 at 1/58 of the FP32 rate):
// magnitudes compare as their bit patterns, and a value's 49-bit fixed-point
// image F = trunc(|a| 2^(49-E)) is its 53-bit significand shifted right by
// E - e + 3 (e its unbiased exponent); the digits are F's 7-bit groups.
__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// E with max|a| / 2^E in [0.5, 1) from the largest magnitude's bit pattern (0 for zero)
__device__ __forceinline__ int oz_exponent_bits(unsigned long long maxbits) {
  if (maxbits == 0) return 0;
  const int ef = (int)(maxbits >> 52);
  if (ef == 0) return -1010 - __clzll((long long)maxbits);  // subnormal: top bit p = 63 - clz, E = p - 1073
  return ef - 1022;
}

template <typename Store>
__device__ __forceinline__ void oz_digits(double v, int E, Store store) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int ef = (int)((bits >> 52) & 0x7ff);
  const unsigned long long frac = bits & 0xfffffffffffffull;
  const unsigned long long M = ef ? (frac | (1ull << 52)) : frac;  // |v| = M 2^(e - 52)
  const int e = ef ? ef - 1023 : -1022;
  const int sh = E - e + 3;  // >= 4 for normal v; a subnormal group may need a left shift
  const unsigned long long F = (M == 0 || sh >= 64) ? 0ull : (sh >= 0 ? (M >> sh) : (M << -sh));
  const bool neg = (bits >> 63) != 0;
#pragma unroll
  for (int s = 0; s < kOzSlices; ++s) {
    const int d = (int)((F >> (42 - 7 * s)) & 127ull);
    store(s, __int2bfloat16_rn(neg ? -d : d));
  }
}

__global__ void oz_slice_rows_kernel(const double *A, long long rpb, long long bstride, long long si, long long sq,
                                     long long rows, int cols, __nv_bfloat16 *out, long long ld_out,
                                     long long sstride, int *exps) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  const double *row = A + (i / rpb) * bstride + (i % rpb) * si;
  unsigned long long mb = 0;
  for (int q = 0; q < cols; ++q) mb = max(mb, abs_bits(row[q * sq]));
  const int E = oz_exponent_bits(mb);
  exps[i] = E;
  __nv_bfloat16 *o = out + i * ld_out;
  for (int q = 0; q < cols; ++q)
    oz_digits(row[q * sq], E, [&](int s, __nv_bfloat16 d) { o[s * sstride + q] = d; });
}

// The same slicing with 16-byte digit stores: a thread packs the digits of 8
// consecutive columns of its row into one 16-byte store per slice (7 stores
// per 8 columns instead of 56 two-byte stores, each of which made the warp
// touch 32 separate sectors).  Needs cols, ld_out and the slice stride to be
// multiples of 8 and a 16-byte aligned output (checked by the launcher).
__global__ void oz_slice_rows8_kernel(const double *A, long long rpb, long long bstride, long long si, long long sq,
                                      long long rows, int cols, __nv_bfloat16 *out, long long ld_out,
                                      long long sstride, int *exps) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  const double *row = A + (i / rpb) * bstride + (i % rpb) * si;
  unsigned long long mb = 0;
  for (int q = 0; q < cols; ++q) mb = max(mb, abs_bits(row[q * sq]));
  const int E = oz_exponent_bits(mb);
  exps[i] = E;
  __nv_bfloat16 *o = out + i * ld_out;
  for (int q0 = 0; q0 < cols; q0 += 8) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = row[(q0 + u) * sq];
    __align__(16) __nv_bfloat16 d[kOzSlices][8];
#pragma unroll
    for (int u = 0; u < 8; ++u) oz_digits(v[u], E, [&](int sl, __nv_bfloat16 x) { d[sl][u] = x; });
#pragma unroll
    for (int sl = 0; sl < kOzSlices; ++sl)
      *reinterpret_cast<uint4 *>(o + sl * sstride + q0) = *reinterpret_cast<const uint4 *>(d[sl]);
  }
}

cudaError_t launch_oz_slice_rows(const double *A, long long rpb, long long bstride, long long si, long long sq,
                                 long long rows, int cols, __nv_bfloat16 *out, long long ld_out,
                                 long long slice_stride, int *exps, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  const bool a16 = ((uintptr_t)out & 15) == 0 && cols % 8 == 0 && ld_out % 8 == 0 && slice_stride % 8 == 0;
  if (a16) {
    HODLR_LAUNCH(oz_slice_rows8_kernel, ceil_div(rows, 128), 128, 0, s, A, rpb, bstride, si, sq, rows, cols, out,
                 ld_out, slice_stride, exps);
    return cudaGetLastError();
  }
  HODLR_LAUNCH(oz_slice_rows_kernel, ceil_div(rows, 128), 128, 0, s, A, rpb, bstride, si, sq, rows, cols, out,
               ld_out, slice_stride, exps);
  return cudaGetLastError();
}

// one warp per (64-row chunk, column).  The value sliced is X (if given)
// plus the FP32 correction add (if given); with xout it is also stored.
__global__ void oz_slice_cols_kernel(const double *X, long long ldx, long long nchunk, int c, __nv_bfloat16 *out,
                                     long long ld_out, long long sstride, int *exps, const int *skip,
                                     const float *add, double *xout) {
  if (skip && *skip) return;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nchunk * c) return;
  const long long ch = w / c;
  const int j = (int)(w % c);
  const long long i0 = ch * kOzChunk + lane, i1 = i0 + 32;
  double v0 = X ? X[i0 + j * ldx] : 0.0, v1 = X ? X[i1 + j * ldx] : 0.0;
  if (add) {
    v0 += (double)add[i0 + j * ldx];
    v1 += (double)add[i1 + j * ldx];
  }
  if (xout) {
    xout[i0 + j * ldx] = v0;
    xout[i1 + j * ldx] = v1;
  }
  unsigned long long mb = max(abs_bits(v0), abs_bits(v1));
#pragma unroll
  for (int o = 16; o; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  const int E = oz_exponent_bits(mb);
  if (lane == 0) exps[ch * c + j] = E;
  __nv_bfloat16 *o = out + j * ld_out;
  oz_digits(v0, E, [&](int s, __nv_bfloat16 d) { o[s * sstride + i0] = d; });
  oz_digits(v1, E, [&](int s, __nv_bfloat16 d) { o[s * sstride + i1] = d; });
}

// The same slicing with 16-byte accesses: 8 lanes per (64-row chunk,
// column), 8 consecutive rows per lane -- four 16-byte loads of X, two of the
// correction, four 16-byte stores of the updated iterate and one per digit
// slice (8 digits), instead of 2-byte digit stores.  Needs 16-byte aligned
// rows (checked by the launcher).
__global__ void oz_slice_cols8_kernel(const double *X, long long ldx, long long nchunk, int c, __nv_bfloat16 *out,
                                      long long ld_out, long long sstride, int *exps, const int *skip,
                                      const float *add, double *xout) {
  static_assert(kOzChunk == 64, "8 lanes x 8 rows per exponent group");
  if (skip && *skip) return;
  const long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const int lane = threadIdx.x & 31, sub = lane & 7;
  if (g >= nchunk * c) return;  // whole 8-lane groups leave together
  const unsigned gmask = 0xffu << (lane & 24);
  const long long ch = g / c;
  const int j = (int)(g % c);
  const long long i0 = ch * kOzChunk + 8 * sub;
  double v[8];
  if (X) {
    const double2 *xp = reinterpret_cast<const double2 *>(X + i0 + j * ldx);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const double2 t = xp[u];
      v[2 * u] = t.x;
      v[2 * u + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = 0.0;
  }
  if (add) {
    const float4 *ap = reinterpret_cast<const float4 *>(add + i0 + j * ldx);
    const float4 a0 = ap[0], a1 = ap[1];
    const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] += (double)av[u];
  }
  if (xout) {
    double2 *op = reinterpret_cast<double2 *>(xout + i0 + j * ldx);
#pragma unroll
    for (int u = 0; u < 4; ++u) op[u] = make_double2(v[2 * u], v[2 * u + 1]);
  }
  unsigned long long mb = 0;
#pragma unroll
  for (int u = 0; u < 8; ++u) mb = max(mb, abs_bits(v[u]));
#pragma unroll
  for (int o = 4; o; o >>= 1) mb = max(mb, __shfl_xor_sync(gmask, mb, o));
  const int E = oz_exponent_bits(mb);
  if (sub == 0) exps[ch * c + j] = E;
  __align__(16) __nv_bfloat16 d[kOzSlices][8];
#pragma unroll
  for (int u = 0; u < 8; ++u) oz_digits(v[u], E, [&](int sl, __nv_bfloat16 x) { d[sl][u] = x; });
  __nv_bfloat16 *o = out + j * ld_out + i0;
#pragma unroll
  for (int sl = 0; sl < kOzSlices; ++sl)
    *reinterpret_cast<uint4 *>(o + sl * sstride) = *reinterpret_cast<const uint4 *>(d[sl]);
}

cudaError_t launch_oz_slice_cols(const double *X, long long ldx, long long n, int c, __nv_bfloat16 *out,
                                 long long ld_out, long long slice_stride, int *exps, const int *skip,
                                 cudaStream_t s, const float *add, double *xout) {
  if (n <= 0 || c <= 0) return cudaSuccess;
  if (n % kOzChunk) return cudaErrorInvalidValue;
  const bool a16 = ((uintptr_t)X & 15) == 0 && ((uintptr_t)add & 15) == 0 && ((uintptr_t)xout & 15) == 0 &&
                   ((uintptr_t)out & 15) == 0 && ldx % 4 == 0 && ld_out % 8 == 0 && slice_stride % 8 == 0;
  if (a16) {
    const long long groups = (n / kOzChunk) * c;
    HODLR_LAUNCH(oz_slice_cols8_kernel, ceil_div(groups * 8, 256), 256, 0, s, X, ldx, n / kOzChunk, c, out,
                 ld_out, slice_stride, exps, skip, add, xout);
    return cudaGetLastError();
  }
  const long long warps = (n / kOzChunk) * c;
  HODLR_LAUNCH(oz_slice_cols_kernel, ceil_div(warps * 32, 256), 256, 0, s, X, ldx, n / kOzChunk, c, out, ld_out,
               slice_stride, exps, skip, add, xout);
  return cudaGetLastError();
}

// one warp per (block, column): T'_b(:, j) = scale .* T_{b^1}(:, j), r <= 64
__global__ void oz_slice_tprime_kernel(const double *T, const double *scale, int r, int k, int nb,
                                       __nv_bfloat16 *out, int *exps, const int *skip) {
  if (skip && *skip) return;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= (long long)nb * k) return;
  const int b = (int)(w / k), j = (int)(w % k);
  const double *src = T + (long long)(b ^ 1) * r * k + (long long)j * r;
  double v[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int q = lane + 32 * h;
    v[h] = q < r ? (scale ? scale[q] : 1.0) * src[q] : 0.0;
  }
  unsigned long long mb = max(abs_bits(v[0]), abs_bits(v[1]));
#pragma unroll
  for (int o = 16; o; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  const int E = oz_exponent_bits(mb);
  if (lane == 0) exps[(long long)b * k + j] = E;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int q = lane + 32 * h;
    if (q < r)
      oz_digits(v[h], E, [&](int s, __nv_bfloat16 d) {
        out[(((long long)b * kOzSlices + s) * k + j) * r + q] = d;
      });
  }
}

cudaError_t launch_oz_slice_tprime(const double *T, const double *scale, int r, int k, int nb, __nv_bfloat16 *out,
                                   int *exps, const int *skip, cudaStream_t s) {
  if (nb <= 0 || k <= 0) return cudaSuccess;
  if (r > 64) return cudaErrorInvalidValue;
  const long long warps = (long long)nb * k;
  HODLR_LAUNCH(oz_slice_tprime_kernel, ceil_div(warps * 32, 256), 256, 0, s, T, scale, r, k, nb, out, exps, skip);
  return cudaGetLastError();
}

// Every level at once: warp w of level l (w < nb(l) k) slices T'_b(:, j) of
// that level; levels found from the warp prefix sums.
__global__ void oz_slice_tprime_all_kernel(const double *T, int r, int k, __nv_bfloat16 *out, int *exps,
                                           TprimeLevels a, const int *skip) {
  if (skip && *skip) return;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= a.wpre[a.L]) return;
  int l = 0;
  while (w >= a.wpre[l + 1]) ++l;
  const long long wl = w - a.wpre[l];
  const int b = (int)(wl / k), j = (int)(wl % k);
  const double *src = T + a.toff[l] + (long long)(b ^ 1) * r * k + (long long)j * r;
  const double *scale = a.scale[l];
  double v[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int q = lane + 32 * h;
    v[h] = q < r ? (scale ? scale[q] : 1.0) * src[q] : 0.0;
  }
  unsigned long long mb = max(abs_bits(v[0]), abs_bits(v[1]));
#pragma unroll
  for (int o = 16; o; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  const int E = oz_exponent_bits(mb);
  if (lane == 0) exps[a.eoff[l] + (long long)b * k + j] = E;
  __nv_bfloat16 *o = out + a.ooff[l];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int q = lane + 32 * h;
    if (q < r)
      oz_digits(v[h], E, [&](int s, __nv_bfloat16 d) { o[(((long long)b * kOzSlices + s) * k + j) * r + q] = d; });
  }
}

// The same with G = r / 8 lanes per (block, column), 8 consecutive ranks per
// lane: 16-byte loads of T (and of the scales) and one 16-byte store per
// digit slice (r a multiple of 8 up to 64; G = 4 or 8).
template <int G>
__global__ void oz_slice_tprime_all8_kernel(const double *T, int r, int k, __nv_bfloat16 *out, int *exps,
                                            TprimeLevels a, const int *skip) {
  if (skip && *skip) return;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int lane = threadIdx.x & 31, sub = lane % G;
  if (w >= a.wpre[a.L]) return;  // whole groups leave together
  const unsigned gmask = (G == 8 ? 0xffu : 0xfu) << (lane & ~(G - 1));
  int l = 0;
  while (w >= a.wpre[l + 1]) ++l;
  const long long wl = w - a.wpre[l];
  const int b = (int)(wl / k), j = (int)(wl % k);
  const int q0 = 8 * sub;
  const double *src = T + a.toff[l] + (long long)(b ^ 1) * r * k + (long long)j * r + q0;
  const double *scale = a.scale[l];
  double v[8];
  if (q0 < r) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const double2 t = reinterpret_cast<const double2 *>(src)[u];
      v[2 * u] = t.x;
      v[2 * u + 1] = t.y;
    }
    if (scale) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const double2 sc = reinterpret_cast<const double2 *>(scale + q0)[u];
        v[2 * u] *= sc.x;
        v[2 * u + 1] *= sc.y;
      }
    }
  } else {
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = 0.0;
  }
  unsigned long long mb = 0;
#pragma unroll
  for (int u = 0; u < 8; ++u) mb = max(mb, abs_bits(v[u]));
#pragma unroll
  for (int o = G / 2; o; o >>= 1) mb = max(mb, __shfl_xor_sync(gmask, mb, o));
  const int E = oz_exponent_bits(mb);
  if (sub == 0) exps[a.eoff[l] + (long long)b * k + j] = E;
  if (q0 >= r) return;
  __align__(16) __nv_bfloat16 d[kOzSlices][8];
#pragma unroll
  for (int u = 0; u < 8; ++u) oz_digits(v[u], E, [&](int sl, __nv_bfloat16 x) { d[sl][u] = x; });
  __nv_bfloat16 *o = out + a.ooff[l];
#pragma unroll
  for (int sl = 0; sl < kOzSlices; ++sl)
    *reinterpret_cast<uint4 *>(o + (((long long)b * kOzSlices + sl) * k + j) * r + q0) =
        *reinterpret_cast<const uint4 *>(d[sl]);
}

cudaError_t launch_oz_slice_tprime_all(const double *T, int r, int k, int L, const int *lev_nb,
                                       const double *const *scale, __nv_bfloat16 *out, int *exps, const int *skip,
                                       cudaStream_t s) {
  if (L <= 0 || k <= 0) return cudaSuccess;
  if (r > 64 || L > kOzMaxLevels) return cudaErrorInvalidValue;
  TprimeLevels a{};
  a.L = L;
  long long w = 0, t = 0, o = 0, e = 0;
  for (int l = 0; l < L; ++l) {
    a.wpre[l] = w;
    a.toff[l] = t;
    a.ooff[l] = o;
    a.eoff[l] = e;
    a.scale[l] = scale[l];
    w += (long long)lev_nb[l] * k;
    t += (long long)lev_nb[l] * r * k;
    o += (long long)lev_nb[l] * kOzSlices * k * r;
    e += (long long)lev_nb[l] * k;
  }
  a.wpre[L] = w;
  bool a16 = r % 8 == 0 && ((uintptr_t)T & 15) == 0 && ((uintptr_t)out & 15) == 0;
  for (int l = 0; l < L && a16; ++l) a16 = ((uintptr_t)scale[l] & 15) == 0;
  if (a16 && r <= 32) {
    HODLR_LAUNCH(oz_slice_tprime_all8_kernel<4>, (unsigned)ceil_div(w * 4, 256), 256, 0, s, T, r, k, out, exps, a,
                 skip);
  } else if (a16) {
    HODLR_LAUNCH(oz_slice_tprime_all8_kernel<8>, (unsigned)ceil_div(w * 8, 256), 256, 0, s, T, r, k, out, exps, a,
                 skip);
  } else {
    HODLR_LAUNCH(oz_slice_tprime_all_kernel, (unsigned)ceil_div(w * 32, 256), 256, 0, s, T, r, k, out, exps, a,
                 skip);
  }
  return cudaGetLastError();
}

// --------------------------------------------------------------- MMA core
__device__ __forceinline__ unsigned ld32(const __nv_bfloat16 *p) { return *reinterpret_cast<const unsigned *>(p); }

__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(smem)), "l"(gmem), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const __nv_bfloat16 *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2(unsigned (&r)[2], const __nv_bfloat16 *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(smem_u32(p)));
}

// acc[d][nt] += sum over digit pairs s + t = d of A_s (16 rows from arow0)
// times B_t (NT column groups of 8 from bcol0, NT = 1 or 2), one 16-wide k
// step at k0.  Tiles: A slice s row i at sA + s * aslice + i * ST, B slice t
// column j at sB + t * bslice + j * ST (k contiguous).  Fragments come from
// ldmatrix: lane L addresses row (L & 7) of 8 x 8 matrix L >> 3, which gives
// the layouts listed at the top of this file.
template <int NT, int ST>
__device__ __forceinline__ void oz_mma_step(float (&acc)[kOzSlices][NT][4], const __nv_bfloat16 *sA, int aslice,
                                            int arow0, const __nv_bfloat16 *sB, int bslice, int bcol0, int k0,
                                            int lane) {
  static_assert(NT == 1 || NT == 2, "one or two column groups");
  unsigned a[kOzSlices][4];
  const int arow = arow0 + (lane & 7) + ((lane >> 3) & 1) * 8, acol = k0 + ((lane >> 4) & 1) * 8;
#pragma unroll
  for (int s = 0; s < kOzSlices; ++s) ldsm_x4(a[s], sA + s * aslice + arow * ST + acol);
  const int brow = bcol0 + (lane & 7) + (NT == 2 ? ((lane >> 4) & 1) * 8 : 0), bcol = k0 + ((lane >> 3) & 1) * 8;
#pragma unroll
  for (int tt = 0; tt < kOzSlices; ++tt) {
    unsigned b[NT][2];
    if constexpr (NT == 2) {
      unsigned q[4];
      ldsm_x4(q, sB + tt * bslice + brow * ST + bcol);
      b[0][0] = q[0];
      b[0][1] = q[1];
      b[1][0] = q[2];
      b[1][1] = q[3];
    } else {
      unsigned q[2];
      ldsm_x2(q, sB + tt * bslice + brow * ST + bcol);
      b[0][0] = q[0];
      b[0][1] = q[1];
    }
#pragma unroll
    for (int s = 0; s + tt < kOzSlices; ++s)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) mma_bf16(acc[s + tt][nt], a[s], b[nt][0], b[nt][1]);
  }
}

__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// sum_d v[d] 2^(-7d) (exact terms) as a normalised double-word
__device__ __forceinline__ void oz_combine(const float (&v)[kOzSlices], float &sh, float &sl) {
  sh = v[0];
  sl = 0.f;
  float w = 1.f;
#pragma unroll
  for (int d = 1; d < kOzSlices; ++d) {
    w *= 0.0078125f;  // 2^-7, exact
    float s, e;
    two_sum_f(sh, v[d] * w, s, e);
    sh = s;
    sl += e;
  }
  const float s = sh + sl;
  sl = sl - (s - sh);
  sh = s;
}

// (ah, al) += (bh, bl)
__device__ __forceinline__ void dw_acc(float &ah, float &al, float bh, float bl) {
  float s, e;
  two_sum_f(ah, bh, s, e);
  e += al + bl;
  ah = s + e;
  al = e - (ah - s);
}

// c - (sh, sl)
__device__ __forceinline__ float2 dw_minus(float2 c, float sh, float sl) {
  float s, e;
  two_sum_f(c.x, -sh, s, e);
  e += c.y - sl;
  const float rh = s + e;
  return make_float2(rh, e - (rh - s));
}

__device__ __forceinline__ float2 split_fp64(double a) {
  const float h = __double2float_rn(a);
  return make_float2(h, __double2float_rn(a - (double)h));
}

// -------------------------------------------------------------- update
// R2_b -= U_b T'_b.  A work item is (child b, 64-row tile); a CTA walks a
// contiguous run of items for one 32-column tile with a two-stage cp.async
// pipeline (the U digits and T'_b digits of item i+1 load while item i is
// multiplied).  8 warps of 16 x 16 outputs.
template <int KP>
__device__ __forceinline__ void oz_update_stage(__nv_bfloat16 *st, const __nv_bfloat16 *Usl, long long uslice,
                                                int r, const __nv_bfloat16 *Tsl, int k, long long rows, int nrt,
                                                long long item, int j0, int tid) {
  constexpr int ST = KP + 8, BM = 64, BN = 32, KC = KP / 8;
  __nv_bfloat16 *sA = st, *sB = st + kOzSlices * BM * ST;
  const long long b = item / nrt;
  const long long row0 = b * rows + (item % nrt) * BM;
  for (int e = tid; e < kOzSlices * BM * KC; e += 256) {
    const int kc = e % KC, i = (e / KC) % BM, s = e / (KC * BM);
    const int kq = kc * 8;
    cp_async16(sA + (s * BM + i) * ST + kq, Usl + s * uslice + (row0 + i) * r + (kq < r ? kq : 0), kq < r ? 16 : 0);
  }
  for (int e = tid; e < kOzSlices * BN * KC; e += 256) {
    const int kc = e % KC, jj = (e / KC) % BN, s = e / (KC * BN);
    const int kq = kc * 8, j = j0 + jj;
    const bool in = kq < r && j < k;
    cp_async16(sB + (s * BN + jj) * ST + kq,
               Tsl + ((b * kOzSlices + s) * k + (in ? j : 0)) * r + (in ? kq : 0), in ? 16 : 0);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <int KP>
__global__ void __launch_bounds__(256) oz_update_kernel(const __nv_bfloat16 *__restrict__ Usl, long long uslice,
                                                        const int *__restrict__ Uexp, int r,
                                                        const __nv_bfloat16 *__restrict__ Tsl,
                                                        const int *__restrict__ Texp, int k, long long rows,
                                                        int nrt, long long items, long long per, float2 *R2,
                                                        long long ldr, const int *skip) {
  if (skip && *skip) return;
  constexpr int ST = KP + 8, BM = 64, BN = 32, STAGE = kOzSlices * (BM + BN) * ST;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *stages = reinterpret_cast<__nv_bfloat16 *>(smem_raw);  // 2 x [A: S x BM x ST | B: S x BN x ST]
  const int j0 = blockIdx.y * BN;
  const long long it0 = (long long)blockIdx.x * per, it1 = min(items, it0 + per);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int wr = (warp & 3) * 16, wc = (warp >> 2) * 16;
  if (it0 >= it1) return;
  oz_update_stage<KP>(stages, Usl, uslice, r, Tsl, k, rows, nrt, it0, j0, tid);
  for (long long it = it0; it < it1; ++it) {
    const int buf = (int)((it - it0) & 1);
    if (it + 1 < it1) {
      oz_update_stage<KP>(stages + (buf ^ 1) * STAGE, Usl, uslice, r, Tsl, k, rows, nrt, it + 1, j0, tid);
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncthreads();
    const long long b = it / nrt;
    const long long row0 = b * rows + (it % nrt) * BM;
    // the R2 values this thread updates, loaded while the products run
    float2 cur[2][4];
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int j = j0 + wc + nt * 8 + 2 * t + (c & 1);
        const long long i = row0 + wr + g + (c >= 2 ? 8 : 0);
        cur[nt][c] = j < k ? R2[i + (long long)j * ldr] : make_float2(0.f, 0.f);
      }
    const __nv_bfloat16 *sA = stages + buf * STAGE, *sB = sA + kOzSlices * BM * ST;
    float acc[kOzSlices][2][4];
#pragma unroll
    for (int d = 0; d < kOzSlices; ++d)
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[d][nt][c] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < KP; k0 += 16) oz_mma_step<2, ST>(acc, sA, BM * ST, wr, sB, BN * ST, wc, k0, lane);
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int j = j0 + wc + nt * 8 + 2 * t + (c & 1);
        if (j >= k) continue;
        const long long i = row0 + wr + g + (c >= 2 ? 8 : 0);
        float v[kOzSlices];
#pragma unroll
        for (int d = 0; d < kOzSlices; ++d) v[d] = acc[d][nt][c];
        float sh, sl;
        oz_combine(v, sh, sl);
        const int ex = Uexp[i] + Texp[b * k + j] - 14;
        R2[i + (long long)j * ldr] = dw_minus(cur[nt][c], ldexpf(sh, ex), ldexpf(sl, ex));
      }
    __syncthreads();  // this stage's buffer is refilled two items later
  }
}

template <int KP>
static cudaError_t oz_update_launch(const __nv_bfloat16 *Usl, long long uslice, const int *Uexp, int r,
                                    const __nv_bfloat16 *Tsl, const int *Texp, int k, long long rows, int nb,
                                    float2 *R2, long long ldr, const int *skip, cudaStream_t s) {
  const int nrt = (int)(rows / 64);
  const long long items = (long long)nrt * nb;
  const int ctiles = ceil_div(k, 32);
  const long long want = std::max<long long>(1, 2 * 152 / ctiles);  // two resident CTAs per SM
  const long long per = std::max<long long>(1, ceil_div(items, want));
  const long long nctas = ceil_div(items, per);
  const size_t bytes = sizeof(__nv_bfloat16) * 2 * kOzSlices * (64 + 32) * (KP + 8);
  auto kern = oz_update_kernel<KP>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  HODLR_LAUNCH(kern, dim3((unsigned)nctas, ctiles), 256, bytes, s, Usl, uslice, Uexp, r, Tsl, Texp, k, rows, nrt,
               items, per, R2, ldr, skip);
  return cudaGetLastError();
}

cudaError_t launch_oz_update(const __nv_bfloat16 *Usl, long long uslice, const int *Uexp, int r,
                             const __nv_bfloat16 *Tsl, const int *Texp, int k, long long rows, int nb, float2 *R2,
                             long long ldr, const int *skip, cudaStream_t s) {
  if (nb <= 0 || k <= 0 || rows <= 0) return cudaSuccess;
  if (rows % 64 || r < 8 || r > 64 || r % 8) return cudaErrorInvalidValue;
  if (r <= 32) return oz_update_launch<32>(Usl, uslice, Uexp, r, Tsl, Texp, k, rows, nb, R2, ldr, skip, s);
  return oz_update_launch<64>(Usl, uslice, Uexp, r, Tsl, Texp, k, rows, nb, R2, ldr, skip, s);
}

// ---------------------------------------------------------------- leaf
// R2 = split(B) - D X per leaf.  A work item is (leaf, 64-row tile) for one
// 32-column tile; its K = m runs in 32-row stages through a two-stage
// cp.async pipeline that continues across the CTA's items; every 64-row
// exponent chunk of X is folded into the double-word sum separately.
__device__ __forceinline__ void oz_leaf_stage(__nv_bfloat16 *st, const __nv_bfloat16 *Dsl, int m,
                                              const __nv_bfloat16 *Xsl, long long n, int k, long long row0,
                                              long long lrow0, int kq0, int j0, int tid) {
  constexpr int ST = 40, BM = 64, BN = 32, KC = 4;
  __nv_bfloat16 *sA = st, *sB = st + kOzSlices * BM * ST;
  for (int e = tid; e < kOzSlices * BM * KC; e += 256) {
    const int kc = e % KC, i = (e / KC) % BM, s = e / (KC * BM);
    cp_async16(sA + (s * BM + i) * ST + kc * 8, Dsl + s * n * m + (row0 + i) * m + kq0 + kc * 8, 16);
  }
  for (int e = tid; e < kOzSlices * BN * KC; e += 256) {
    const int kc = e % KC, jj = (e / KC) % BN, s = e / (KC * BN);
    const int j = j0 + jj;
    const bool in = j < k;
    cp_async16(sB + (s * BN + jj) * ST + kc * 8,
               Xsl + s * n * k + (long long)(in ? j : 0) * n + lrow0 + kq0 + kc * 8, in ? 16 : 0);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__global__ void __launch_bounds__(256) oz_leaf_kernel(const __nv_bfloat16 *__restrict__ Dsl,
                                                      const int *__restrict__ Dexp, int m,
                                                      const __nv_bfloat16 *__restrict__ Xsl,
                                                      const int *__restrict__ Xexp, long long n, int k,
                                                      const double *__restrict__ B, long long ldb, float2 *R2,
                                                      long long ldr, int nrt, long long items, long long per,
                                                      const int *skip) {
  if (skip && *skip) return;
  constexpr int ST = 40, BM = 64, BN = 32, STAGE = kOzSlices * (BM + BN) * ST;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *stages = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
  const int j0 = blockIdx.y * BN;
  const long long it0 = (long long)blockIdx.x * per, it1 = min(items, it0 + per);
  if (it0 >= it1) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int wr = (warp & 3) * 16, wc = (warp >> 2) * 16;
  const int spi = m / 32;  // stages per item
  const long long nst = (it1 - it0) * spi;
  auto stage_of = [&](long long q, long long &row0, long long &lrow0, int &kq0) {
    const long long it = it0 + q / spi;
    kq0 = (int)(q % spi) * 32;
    lrow0 = (it / nrt) * m;
    row0 = lrow0 + (it % nrt) * BM;
  };
  {
    long long row0, lrow0;
    int kq0;
    stage_of(0, row0, lrow0, kq0);
    oz_leaf_stage(stages, Dsl, m, Xsl, n, k, row0, lrow0, kq0, j0, tid);
  }
  float rh[2][4], rl[2][4], acc[kOzSlices][2][4];
  for (long long q = 0; q < nst; ++q) {
    const int buf = (int)(q & 1);
    if (q + 1 < nst) {
      long long row0, lrow0;
      int kq0;
      stage_of(q + 1, row0, lrow0, kq0);
      oz_leaf_stage(stages + (buf ^ 1) * STAGE, Dsl, m, Xsl, n, k, row0, lrow0, kq0, j0, tid);
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncthreads();
    long long row0, lrow0;
    int kq0;
    stage_of(q, row0, lrow0, kq0);
    if (kq0 == 0) {
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int c = 0; c < 4; ++c) rh[nt][c] = rl[nt][c] = 0.f;
    }
    if ((kq0 & 63) == 0) {
#pragma unroll
      for (int d = 0; d < kOzSlices; ++d)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
          for (int c = 0; c < 4; ++c) acc[d][nt][c] = 0.f;
    }
    const __nv_bfloat16 *sA = stages + buf * STAGE, *sB = sA + kOzSlices * BM * ST;
#pragma unroll
    for (int k0 = 0; k0 < 32; k0 += 16) oz_mma_step<2, ST>(acc, sA, BM * ST, wr, sB, BN * ST, wc, k0, lane);
    if ((kq0 & 63) == 32) {  // a 64-row exponent chunk of X is complete
      const long long xch = (lrow0 + kq0 - 32) / kOzChunk;
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int j = j0 + wc + nt * 8 + 2 * t + (c & 1);
          if (j >= k) continue;
          const long long i = row0 + wr + g + (c >= 2 ? 8 : 0);
          float v[kOzSlices];
#pragma unroll
          for (int d = 0; d < kOzSlices; ++d) v[d] = acc[d][nt][c];
          float sh, sl;
          oz_combine(v, sh, sl);
          const int ex = Dexp[i] + Xexp[xch * k + j] - 14;
          dw_acc(rh[nt][c], rl[nt][c], ldexpf(sh, ex), ldexpf(sl, ex));
        }
    }
    if (kq0 + 32 == m) {  // the item's last stage: R2 = split(B) - D X
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int j = j0 + wc + nt * 8 + 2 * t + (c & 1);
          if (j >= k) continue;
          const long long i = row0 + wr + g + (c >= 2 ? 8 : 0);
          R2[i + (long long)j * ldr] = dw_minus(split_fp64(B[i + (long long)j * ldb]), rh[nt][c], rl[nt][c]);
        }
    }
    __syncthreads();
  }
}

cudaError_t launch_oz_leaf(const __nv_bfloat16 *Dsl, const int *Dexp, int m, int nleaf, const __nv_bfloat16 *Xsl,
                           const int *Xexp, long long n, int k, const double *B, long long ldb, float2 *R2,
                           long long ldr, const int *skip, cudaStream_t s) {
  if (nleaf <= 0 || k <= 0) return cudaSuccess;
  if (m % 64) return cudaErrorInvalidValue;
  const int nrt = m / 64, ctiles = ceil_div(k, 32);
  const long long items = (long long)nrt * nleaf;
  const long long want = std::max<long long>(1, 2 * 152 / ctiles);
  const long long per = std::max<long long>(1, ceil_div(items, want));
  const long long nctas = ceil_div(items, per);
  const size_t bytes = sizeof(__nv_bfloat16) * 2 * kOzSlices * (64 + 32) * 40;
  cudaError_t e = cudaFuncSetAttribute(oz_leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  HODLR_LAUNCH(oz_leaf_kernel, dim3((unsigned)nctas, ctiles), 256, bytes, s, Dsl, Dexp, m, Xsl, Xexp, n, k, B, ldb,
               R2, ldr, nrt, items, per, skip);
  return cudaGetLastError();
}

// -------------------------------------------------------------- reduce
// T_b = V_b^T X_b over a range of 64-row chunks.  CTA: (block, chunk group),
// 32 columns; the RT x 32 output is (RT/16) x 4 MMA tiles spread over the
// 8 warps; each chunk's exact diagonal sums are folded into a double-word
// running sum with the chunk's exponents.
static constexpr int kOzRedTarget = 4 * 152;

static void oz_reduce_plan(long long rows, int nb, int k, int &groups, int &per) {
  const long long nch = rows / kOzChunk;
  const long long base = (long long)nb * ceil_div(k, 32);
  long long gr = base >= kOzRedTarget ? 1 : ceil_div(kOzRedTarget, base);
  gr = std::max<long long>(1, std::min<long long>(gr, nch));
  per = (int)ceil_div(nch, gr);
  groups = (int)ceil_div(nch, per);
}

size_t oz_reduce_workspace_doubles(long long rows, int nb, int r, int k) {
  int groups, per;
  oz_reduce_plan(rows, nb, k, groups, per);
  return groups > 1 ? (size_t)nb * groups * r * k : 0;
}

// CTA: (block, chunk group) x 32 columns; the RT x 32 output is (RT/16) x 4
// MMA tiles over the 8 warps.  Each 64-row chunk is staged whole (V and X
// digits), multiplied, and its exact diagonal sums folded into a
// double-word running sum with the chunk's exponents; several resident CTAs
// per SM overlap one another's loads.
template <int RT>
__global__ void __launch_bounds__(256, RT == 64 ? 2 : 3) oz_reduce_kernel(const __nv_bfloat16 *__restrict__ Vsl, long long vslice,
                                                           const int *__restrict__ Vexp, int r,
                                                           const __nv_bfloat16 *__restrict__ Xsl,
                                                           const int *__restrict__ Xexp, long long n, int k,
                                                           long long rows, int groups, int per, double *out,
                                                           const int *skip) {
  if (skip && *skip) return;
  constexpr int KP = kOzChunk, ST = KP + 8, BN = 32, KC = KP / 8;
  constexpr int MT = RT / 16, TILES = MT * 4, TPW = (TILES + 7) / 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smem_raw);  // [S][RT][ST]  (rows = ranks q)
  __nv_bfloat16 *sB = sA + kOzSlices * RT * ST;                      // [S][BN][ST]  (columns j)
  const int grp = blockIdx.x % groups, b = blockIdx.x / groups, j0 = blockIdx.y * BN;
  const long long nch = rows / kOzChunk;
  const long long c_begin = (long long)grp * per, c_end = std::min<long long>(nch, c_begin + per);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  float rh[TPW][4], rl[TPW][4];
#pragma unroll
  for (int u = 0; u < TPW; ++u)
#pragma unroll
    for (int c = 0; c < 4; ++c) rh[u][c] = rl[u][c] = 0.f;
  for (long long ch = c_begin; ch < c_end; ++ch) {
    const long long grow = (long long)b * rows + ch * kOzChunk;  // first row of the chunk
    if (ch != c_begin) __syncthreads();
    for (int e = tid; e < kOzSlices * RT * KC; e += 256) {
      const int kc = e % KC, q = (e / KC) % RT, s = e / (KC * RT);
      const bool in = q < r;
      cp_async16(sA + (s * RT + q) * ST + kc * 8, Vsl + s * vslice + (long long)(in ? q : 0) * n + grow + kc * 8,
                 in ? 16 : 0);
    }
    for (int e = tid; e < kOzSlices * BN * KC; e += 256) {
      const int kc = e % KC, jj = (e / KC) % BN, s = e / (KC * BN);
      const int j = j0 + jj;
      const bool in = j < k;
      cp_async16(sB + (s * BN + jj) * ST + kc * 8, Xsl + s * n * k + (long long)(in ? j : 0) * n + grow + kc * 8,
                 in ? 16 : 0);
    }
    cp_async_wait_all();
    __syncthreads();
    const long long gch = grow / kOzChunk;
#pragma unroll
    for (int u = 0; u < TPW; ++u) {
      const int tile = warp + 8 * u;
      if (tile >= TILES) continue;
      const int mt = tile / 4, nt = tile % 4;
      float acc[kOzSlices][1][4];
#pragma unroll
      for (int d = 0; d < kOzSlices; ++d)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[d][0][c] = 0.f;
#pragma unroll
      for (int k0 = 0; k0 < KP; k0 += 16) oz_mma_step<1, ST>(acc, sA, RT * ST, mt * 16, sB, BN * ST, nt * 8, k0, lane);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int q = mt * 16 + g + (c >= 2 ? 8 : 0), j = j0 + nt * 8 + 2 * t + (c & 1);
        if (q >= r || j >= k) continue;
        float v[kOzSlices];
#pragma unroll
        for (int d = 0; d < kOzSlices; ++d) v[d] = acc[d][0][c];
        float sh, sl;
        oz_combine(v, sh, sl);
        const int ex = Vexp[gch * r + q] + Xexp[gch * k + j] - 14;
        dw_acc(rh[u][c], rl[u][c], ldexpf(sh, ex), ldexpf(sl, ex));
      }
    }
  }
  double *o = out + ((long long)b * groups + grp) * r * k;
#pragma unroll
  for (int u = 0; u < TPW; ++u) {
    const int tile = warp + 8 * u;
    if (tile >= TILES) continue;
    const int mt = tile / 4, nt = tile % 4;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int q = mt * 16 + g + (c >= 2 ? 8 : 0), j = j0 + nt * 8 + 2 * t + (c & 1);
      if (q < r && j < k) o[q + (long long)j * r] = (double)rh[u][c] + (double)rl[u][c];
    }
  }
}

__global__ void oz_pass2_kernel(const double *__restrict__ partial, int groups, long long blk, double *out,
                                const int *skip) {
  if (skip && *skip) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (e >= blk) return;
  const double *p = partial + (long long)b * groups * blk + e;
  double s = 0.0;
  for (int c = 0; c < groups; ++c) s += p[(long long)c * blk];
  out[(long long)b * blk + e] = s;
}

template <int RT>
static cudaError_t oz_reduce_rt(const __nv_bfloat16 *Vsl, long long vslice, const int *Vexp, int r,
                                const __nv_bfloat16 *Xsl, const int *Xexp, long long n, int k, long long rows,
                                int nb, int groups, int per, double *dst, const int *skip, cudaStream_t s) {
  const size_t bytes = sizeof(__nv_bfloat16) * kOzSlices * (RT + 32) * (kOzChunk + 8);
  auto kern = oz_reduce_kernel<RT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)((long long)nb * groups), ceil_div(k, 32));
  HODLR_LAUNCH(kern, grid, 256, bytes, s, Vsl, vslice, Vexp, r, Xsl, Xexp, n, k, rows, groups, per, dst, skip);
  return cudaGetLastError();
}

cudaError_t launch_oz_reduce(const __nv_bfloat16 *Vsl, long long vslice, const int *Vexp, int r,
                             const __nv_bfloat16 *Xsl, const int *Xexp, long long n, int k, long long rows, int nb,
                             double *out, double *work, const int *skip, cudaStream_t s) {
  if (nb <= 0 || k <= 0) return cudaSuccess;
  if (rows % kOzChunk || r < 1 || r > 64) return cudaErrorInvalidValue;
  int groups, per;
  oz_reduce_plan(rows, nb, k, groups, per);
  double *dst = groups > 1 ? work : out;
  cudaError_t e;
  if (r <= 16)
    e = oz_reduce_rt<16>(Vsl, vslice, Vexp, r, Xsl, Xexp, n, k, rows, nb, groups, per, dst, skip, s);
  else if (r <= 32)
    e = oz_reduce_rt<32>(Vsl, vslice, Vexp, r, Xsl, Xexp, n, k, rows, nb, groups, per, dst, skip, s);
  else
    e = oz_reduce_rt<64>(Vsl, vslice, Vexp, r, Xsl, Xexp, n, k, rows, nb, groups, per, dst, skip, s);
  if (e != cudaSuccess) return e;
  if (groups > 1) {
    const long long blk = (long long)r * k;
    HODLR_LAUNCH(oz_pass2_kernel, dim3(ceil_div(blk, 256), nb), 256, 0, s, work, groups, blk, out, skip);
  }
  return cudaGetLastError();
}

}  // namespace hodlr
