// FP64-accurate residual R2 = split(B) - D X - sum_l U_l T'_l on the
// 5th-generation tensor cores (tcgen05, accumulators in tensor memory).
//
// One pass over 128-row tiles: the leaf term and every level's update term
// of a tile accumulate in the registers of the epilogue warps, so the
// double-word residual is written once, not once per level.  The operands
// are the exact 7-bit bf16 digits of the Ozaki splitting (ozaki.cuh): a
// "group" is one exponent-scaled product -- a 64-row chunk of the leaf
// product (A = D digits, scaled per row; B = X digits, scaled per 64-row
// chunk and column) or one level's update (A = U_l digits per row, B = T'_l
// digits per column) -- and its 28 digit pairs (s + t <= 6) accumulate into
// seven per-diagonal FP32 sums, which are exact (at most 7 x 64 products
// below 2^14 each).
//
// CTA (persistent, one per SM): warp 0 streams the digit tiles with TMA
// (64-byte swizzled K-major 32-wide slabs, A 128 x 32, B 64 x 32) through a
// 16-stage ring; one thread of warp 1 issues tcgen05.mma (M 128, N 64,
// K 16, bf16 -> f32) into tensor memory, diagonals 0-3 in one region and
// 4-6 in another so that the epilogue drains one while the next group's
// products fill the other; eight epilogue warps read the sums with
// tcgen05.ld (warp w sees lanes 32 (w % 4) .. + 31, i.e. those rows; warps
// 2-5 take columns 0-31, warps 6-9 columns 32-63), fold them with the
// group's exponents into the double-word running sum and finally write
// R2 = split(B) - sum.  Every wait is bounded: on timeout the kernel
// records HODLR_ERR_TIMEOUT, all roles stop, in-flight products and copies
// are waited for (bounded) and the tensor memory is released.
#include <algorithm>

#include "kernels.cuh"
#include "ozaki.cuh"
#include "tcgen05.cuh"
#include "tma.cuh"

namespace hodlr {

namespace {

constexpr int kRows = 128;   // tile rows (MMA M)
constexpr int kCols = 64;    // tile columns (MMA N)
constexpr int kSlab = 32;    // K per stage: one 64-byte swizzled row
// A stage holds one K-half of a group: the seven A digit slabs (128 x 32
// each) and, after them, the seven B digit slabs (64 x 32 each) contiguous,
// so that one MMA of A slab s against B slabs t0 .. t1 (N up to 256) writes
// each product A_s B_t into the columns of its diagonal s + t.
constexpr int kStages = 2;
constexpr int kABytes = kRows * kSlab * 2;
constexpr int kBBytes = kCols * kSlab * 2;
constexpr int kAAll = kOzSlices * kABytes;
constexpr int kStageBytes = kOzSlices * (kABytes + kBBytes);
constexpr int kEpiWarps = 16;  // four per SM sub-partition; each thread one row, 16 columns
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr int kEpiCols = kCols / (kEpiWarps / 4);
constexpr unsigned kTmemCols = 512;
// kind::f16 instruction descriptor: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr unsigned idesc_n(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) | ((unsigned)(kRows >> 4) << 24);
}
constexpr long long kWaitCycles = 2000000000LL;  // about one second

struct Shared {
  uint64_t full[kStages], empty[kStages];
  uint64_t acc_full[2], acc_empty[2], drain;
  unsigned tmem;
  int abort;
  int consumed;  // stages the MMA thread consumed (for the drain after an abort)
};

__device__ __forceinline__ void arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded wait that also ends when another role has aborted.
__device__ __forceinline__ bool wait_or_abort(uint64_t *bar, unsigned parity, Shared *sh) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*(volatile int *)&sh->abort) return false;
    if (clock64() - t0 > kWaitCycles) {
      *(volatile int *)&sh->abort = 1;
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// 2^e for e in [-126, 127], from its bit pattern
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }

// Running double-word sum (rh, rl) += 2^ex sum_d v[d] 2^(-7 d) for the
// exact diagonal sums v of one group.  Diagonals 0-3 enter through
// error-free two-sums; diagonals 4-6 are at most 2^-5 of a unit of
// diagonal 0 and go straight into rl (rounding 2^-29 of that unit, 2^-52
// of the largest possible leading term); rl is renormalised once per group.
// The scale factors are built from exponent bits: the caller checks that
// ex - 42 .. ex is a normal range (else fold_any).
template <int W>
__device__ __forceinline__ void fold_hi(float &rh, float &rl, const unsigned (&v)[4][W], int c, int ex) {
  float p = pow2f(ex);
#pragma unroll
  for (int d = 0; d < 4; ++d) {
    float s, e;
    two_sum(rh, __uint_as_float(v[d][c]) * p, s, e);
    rh = s;
    rl += e;
    p *= 0.0078125f;  // 2^-7
  }
}
template <int W>
__device__ __forceinline__ void fold_lo(float &rh, float &rl, const unsigned (&v)[3][W], int c, int ex) {
  float p = pow2f(ex - 28);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    rl = fmaf(__uint_as_float(v[d][c]), p, rl);
    p *= 0.0078125f;
  }
  float s, e;
  two_sum(rh, rl, s, e);
  rh = s;
  rl = e;
}
// One accumulator region of this thread's row and 16 columns: diagonals
// D0 .. D0 + ND - 1 at tensor-memory columns tl0 + d * kCols + c, read in
// 4-column chunks with the next chunk's load in flight while the current
// one is folded into (rh, rl).  Warp-uniform `fast`: every scale factor of
// the warp's rows and columns is a normal float.
struct Acc16 {
  float h[16], l[16];
};
// Exponents outside that range: ldexpf scaling (rare; not inlined).
template <int ND, int D0>
__device__ __noinline__ Acc16 drain_any(unsigned tl0, Acc16 acc, int er, int ec) {
  for (int cc = 0; cc < 16; cc += 4) {
    unsigned v[1][ND][4];
#pragma unroll
    for (int d = 0; d < ND; ++d) tc_ld4(tl0 + (unsigned)(d * kCols + cc), v[0][d]);
    tc_wait_ld(v[0]);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int ex = er + __shfl_sync(0xffffffffu, ec, cc + c);
      float rh = acc.h[cc + c], rl = acc.l[cc + c];
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        float s, e;
        two_sum(rh, ldexpf(__uint_as_float(v[0][d][c]), ex - 7 * (D0 + d)), s, e);
        rh = s;
        rl += e;
      }
      float s, e;
      two_sum(rh, rl, s, e);
      acc.h[cc + c] = s;
      acc.l[cc + c] = e;
    }
  }
  return acc;
}

template <int ND, int D0>
__device__ __forceinline__ void drain_region(unsigned tl0, float (&rh)[16], float (&rl)[16], int er, int ec,
                                             bool fast) {
  if (!fast) {
    Acc16 acc;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      acc.h[c] = rh[c];
      acc.l[c] = rl[c];
    }
    acc = drain_any<ND, D0>(tl0, acc, er, ec);
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      rh[c] = acc.h[c];
      rl[c] = acc.l[c];
    }
    return;
  }
  unsigned v[2][ND][4];
#pragma unroll
  for (int d = 0; d < ND; ++d) tc_ld4(tl0 + (unsigned)(d * kCols), v[0][d]);
  tc_wait_ld(v[0]);
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    const int cur = ch & 1;
    if (ch + 1 < 4) {
#pragma unroll
      for (int d = 0; d < ND; ++d) tc_ld4(tl0 + (unsigned)(d * kCols + 4 * (ch + 1)), v[cur ^ 1][d]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int cc = 4 * ch + c, ex = er + __shfl_sync(0xffffffffu, ec, cc);
      if constexpr (D0 == 0)
        fold_hi(rh[cc], rl[cc], v[cur], c, ex);
      else
        fold_lo(rh[cc], rl[cc], v[cur], c, ex);
    }
    if (ch + 1 < 4) tc_wait_ld(v[cur ^ 1]);
  }
}

// (hi, lo) with hi + lo = v to 2^-48 relative: hi the significand rounded
// to 24 bits, lo the exact remainder rounded to FP32 -- from the bit
// pattern, without FP64 arithmetic (normal magnitudes 2^-70 .. 2^100;
// others through FP64 conversions).
__device__ __forceinline__ float2 split_bits(double v) {
  const long long b = __double_as_longlong(v);
  const long long mag = b & 0x7fffffffffffffffLL;
  const int ex = (int)(mag >> 52) - 1023;
  if (mag == 0) return make_float2(0.f, 0.f);
  if (ex < -70 || ex > 100) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
  }
  const long long hb = (mag + (1LL << 28)) & ~((1LL << 29) - 1);  // 24-bit significand, rounded
  const int eh = (int)(hb >> 52) - 1023;
  float hi = __uint_as_float(((unsigned)(eh + 127) << 23) | (unsigned)((hb >> 29) & 0x7fffff));
  float lo = (float)(mag - hb) * pow2f(ex - 52);  // |mag - hb| <= 2^28 units of 2^(ex - 52)
  if (b < 0) {
    hi = -hi;
    lo = -lo;
  }
  return make_float2(hi, lo);
}

}  // namespace

constexpr int kMaxLevels = 32;

// Two products share the pipeline below.  Mode 0, the residual: a work item
// is a 128-row tile x 64 columns; its groups are the leaf term's 64-row
// chunks (A = D digits, B = X digits) and every level with a block over the
// tile (A = U_l digits, B = T'_l digits); R2 is written once per item.
// Mode 1, the reductions T_l = V_l^T X of every level: a work item is a
// range of R rows x a stack of QL = 128 / r levels x 64 columns; A = the
// stacked levels' V digits (row (l, q) = line l r + q of the V digit
// matrix), B = X digits, one group per 64-row chunk of the range.  A level
// block that ends inside the range is written to T when it ends; a block
// longer than the range gets one partial per range, summed by
// oz_tc_pass2_kernel in a fixed order.
struct OzTcArgs {
  // level l: blocks of lrows[l] rows from row 0 (lnb[l] of them)
  long long lrows[kMaxLevels];
  int lnb[kMaxLevels];
  // mode 0: block b's T' digits start at line ltrow[l] + 7 k b, its column
  // exponents at Texp + lteo[l] + k b
  long long ltrow[kMaxLevels], lteo[kMaxLevels];
  // mode 1: level l's T blocks at T + toff[l] (r x k each, ld r), its
  // partials at P + poff[l] ((b parts[l] + part) r k)
  long long toff[kMaxLevels], poff[kMaxLevels];
  int parts[kMaxLevels];
  const int *Dexp, *Xexp, *Uexp, *Texp, *Vexp;
  const double *B;
  long long ldb;
  float2 *R2;
  long long ldr;
  double *T, *P;
  long long n, R;
  int m, L, r, k, QL, nstack;
  long long items;
  int nct;  // column tiles
  const int *skip;
  DevStatus *st;
};

// Group g of the mode-0 tile at row0: the leaf chunks always, level l when a block of it covers the tile.
__device__ __forceinline__ bool has_group(const OzTcArgs &a, int g, int leaf_groups, long long row0) {
  if (g < leaf_groups) return true;
  const int l = g - leaf_groups;
  return row0 < (long long)a.lnb[l] * a.lrows[l];
}

struct ItemGeo {
  long long row0;  // mode 0: the tile's first row; mode 1: the range's
  int j0, stack, g0, g1;
};

template <int MODE>
__device__ __forceinline__ ItemGeo item_geo(const OzTcArgs &a, long long item) {
  ItemGeo it;
  it.j0 = (int)(item % a.nct) * kCols;
  const long long t = item / a.nct;
  if (MODE == 0) {
    it.row0 = t * kRows;
    it.stack = 0;
    it.g0 = 0;
    it.g1 = a.m / 64 + a.L;
  } else {
    it.stack = (int)(t % a.nstack);
    it.row0 = (t / a.nstack) * a.R;
    it.g0 = (int)(it.row0 / 64);
    it.g1 = (int)(std::min<long long>(it.row0 + a.R, a.n) / 64);
  }
  return it;
}

template <int MODE>
__device__ __forceinline__ bool group_exists(const OzTcArgs &a, const ItemGeo &it, int g) {
  return MODE == 1 || has_group(a, g, a.m / 64, it.row0);
}
template <int MODE>
__device__ __forceinline__ int group_khalves(const OzTcArgs &a, int g) {
  return (MODE == 1 || g < a.m / 64) ? 2 : (a.r + kSlab - 1) / kSlab;
}

// Writes 16 columns of this thread's row, as FP64, at out + j * ld (j < k).
__device__ __forceinline__ void store_fp64(double *out, long long ld, const float (&rh)[kEpiCols],
                                           const float (&rl)[kEpiCols], int jb, int k) {
#pragma unroll
  for (int c = 0; c < kEpiCols; ++c)
    if (jb + c < k) out[(long long)(jb + c) * ld] = (double)rh[c] + (double)rl[c];
}

template <int MODE>
__global__ void __launch_bounds__(kThreads, 1)
oz_tc_kernel(const __grid_constant__ CUtensorMap mapA0, const __grid_constant__ CUtensorMap mapB0,
             const __grid_constant__ CUtensorMap mapA1, const __grid_constant__ CUtensorMap mapB1, OzTcArgs a) {
  if (a.skip && *a.skip) return;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *stages =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  Shared *sh = reinterpret_cast<Shared *>(stages + kStages * kStageBytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int leaf_groups = a.m / 64;

  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(&sh->full[i], 1);
      mbar_init(&sh->empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&sh->acc_full[i], 1);
      mbar_init(&sh->acc_empty[i], kEpiWarps);
    }
    mbar_init(&sh->drain, 1);
    sh->abort = 0;
    sh->consumed = 0;
    mbar_fence_init();
  }
  if (warp == 1) {
    tc_alloc(&sh->tmem, kTmemCols);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = sh->tmem;
  long long issued = 0;  // stages issued by the producer thread

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      prefetch_tensormap(&mapA0);
      prefetch_tensormap(&mapB0);
      if (MODE == 0) {
        prefetch_tensormap(&mapA1);
        prefetch_tensormap(&mapB1);
      }
      bool ok = true;
      for (long long item = blockIdx.x; ok && item < a.items; item += gridDim.x) {
        const ItemGeo it = item_geo<MODE>(a, item);
        const long long lrow0 = it.row0 - it.row0 % a.m;
        for (int g = it.g0; ok && g < it.g1; ++g) {
          if (!group_exists<MODE>(a, it, g)) continue;
          const int nkh = group_khalves<MODE>(a, g);
          // slab coordinates of slice 0, K-half 0, and the per-slice line strides
          const CUtensorMap *ma, *mb;
          int ax, bx;
          long long ay, by, as, bs;
          if (MODE == 1) {
            ma = &mapA0;
            mb = &mapB0;
            ax = bx = g * 64;
            ay = (long long)it.stack * a.QL * a.r;
            as = (long long)a.L * a.r;
            by = it.j0;
            bs = a.k;
          } else if (g < leaf_groups) {
            ma = &mapA0;
            mb = &mapB0;
            ax = g * 64;
            ay = it.row0;
            as = a.n;
            bx = (int)(lrow0 + g * 64);
            by = it.j0;
            bs = a.k;
          } else {
            const int l = g - leaf_groups;
            ma = &mapA1;
            mb = &mapB1;
            ax = bx = 0;
            ay = (long long)l * a.n + it.row0;
            as = (long long)a.L * a.n;
            by = a.ltrow[l] + (it.row0 / a.lrows[l]) * kOzSlices * a.k + it.j0;
            bs = a.k;
          }
          for (int kh = 0; ok && kh < nkh; ++kh) {
            const int slot = (int)(issued % kStages);
            if (!wait_or_abort(&sh->empty[slot], (unsigned)(((issued / kStages) & 1) ^ 1), sh)) {
              ok = false;
              break;
            }
            unsigned char *st = stages + slot * kStageBytes;
            mbar_arrive_expect_tx(&sh->full[slot], kStageBytes);
#pragma unroll 1
            for (int sl = 0; sl < kOzSlices; ++sl) {
              tma_load_2d(st + sl * kABytes, ma, &sh->full[slot], ax + kh * kSlab, (int)(ay + sl * as));
              tma_load_2d(st + kAAll + sl * kBBytes, mb, &sh->full[slot], bx + kh * kSlab, (int)(by + sl * bs));
            }
            ++issued;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ----------------------------------------------------------- MMA issue
    if (lane == 0) {
      long long it_s = 0, gcount = 0;
      bool ok = true;
      for (long long item = blockIdx.x; ok && item < a.items; item += gridDim.x) {
        const ItemGeo it = item_geo<MODE>(a, item);
        for (int g = it.g0; ok && g < it.g1; ++g) {
          if (!group_exists<MODE>(a, it, g)) continue;
          const int nkh = group_khalves<MODE>(a, g);
          const unsigned par_empty = (unsigned)((gcount & 1) ^ 1);
          ++gcount;
          // The group's K-halves sit in stages it_s (and it_s + 1).  Each
          // K-half: diagonals 0-3 (tensor-memory columns 0-255, A_s against
          // B_0 .. B_{3-s}), then diagonals 4-6 (columns 256-447, A_s
          // against B_{max(0, 4-s)} .. B_{6-s}); a K-half's stage is released
          // as soon as its products are issued, so that the next group's
          // first K-half loads while the second one multiplies.
          for (int kh = 0; ok && kh < nkh; ++kh) {
            const long long sidx = it_s + kh;
            const int slot = (int)(sidx & (kStages - 1));
            if (!wait_or_abort(&sh->full[slot], (unsigned)((sidx / kStages) & 1), sh)) {
              ok = false;
              break;
            }
            const unsigned sa = smem_u32(stages + slot * kStageBytes);
            const uint64_t adesc = desc_sw64(sa), bdesc = desc_sw64(sa + kAAll);
            if (kh == 0 && !wait_or_abort(&sh->acc_empty[0], par_empty, sh)) {
              ok = false;
              break;
            }
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < kSlab / 16; ++kk)  // +32 bytes = +2 in the descriptor's address field
#pragma unroll
              for (int s = 0; s < 4; ++s)
                tc_mma(tmem + (unsigned)(64 * s), adesc + (uint64_t)(kABytes / 16 * s + 2 * kk),
                       bdesc + (uint64_t)(2 * kk), idesc_n(64 * (4 - s)), (kh > 0 || kk > 0 || s > 0) ? 1u : 0u);
            if (kh == nkh - 1) tc_commit(&sh->acc_full[0]);
            if (kh == 0 && !wait_or_abort(&sh->acc_empty[1], par_empty, sh)) {
              ok = false;
              break;
            }
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < kSlab / 16; ++kk)
#pragma unroll
              for (int s = 0; s < kOzSlices; ++s) {
                const int t0 = s < 4 ? 4 - s : 0;
                tc_mma(tmem + (unsigned)(64 * (s + t0)), adesc + (uint64_t)(kABytes / 16 * s + 2 * kk),
                       bdesc + (uint64_t)(kBBytes / 16 * t0 + 2 * kk), idesc_n(64 * (7 - s - t0)),
                       (kh > 0 || kk > 0 || s > 0) ? 1u : 0u);
              }
            if (kh == nkh - 1) tc_commit(&sh->acc_full[1]);
            tc_commit(&sh->empty[slot]);
          }
          if (!ok) break;
          it_s += nkh;
        }
      }
      sh->consumed = (int)it_s;
      tc_commit(&sh->drain);  // completes once every product issued above has
      if (!wait_or_abort(&sh->drain, 0, sh)) {
        // the products were still running after the bounded wait: keep waiting,
        // bounded, since the tensor memory is freed below
        const long long t0 = clock64();
        while (!mbar_try_wait(&sh->drain, 0) && clock64() - t0 < kWaitCycles) {
        }
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3, cq = (warp - 2) >> 2;
    const int p = 32 * q + lane;  // the thread's row of the product
    const unsigned tl = tmem + ((unsigned)(32 * q) << 16) + (unsigned)(kEpiCols * cq);
    // mode 1: the row is rank qq of stacked level lq
    const int lq = MODE == 1 ? p / a.r : 0, qq = MODE == 1 ? p - lq * a.r : 0;
    long long gcount = 0;
    bool ok = true;
    for (long long item = blockIdx.x; ok && item < a.items; item += gridDim.x) {
      const ItemGeo it = item_geo<MODE>(a, item);
      const long long i = it.row0 + p;  // mode 0: the thread's matrix row
      const int jb = it.j0 + kEpiCols * cq;
      const int jl = jb + (lane & (kEpiCols - 1));  // lane c holds column jb + c's exponent
      const long long lrow0 = it.row0 - it.row0 % a.m;
      const int l1 = it.stack * a.QL + lq;          // mode 1: the row's level
      const bool valid = MODE == 0 || (lq < a.QL && l1 < a.L);
      // a warp whose rows are all padding of the last level stack only keeps
      // the barrier phases (waits for the products, then releases them)
      const bool idle = MODE == 1 && __all_sync(0xffffffffu, !valid);
      const long long rows1 = (MODE == 1 && valid) ? a.lrows[l1] : 0;
      // the row exponent of this thread's row and the column exponent of
      // column jl in group g (loaded one group ahead of their use)
      auto exps = [&](int g, int &erow, int &ec) {
        const int *ecol;
        if (MODE == 1) {
          erow = valid ? a.Vexp[((long long)l1 * (a.n / kOzChunk) + g) * a.r + qq] : 0;
          ecol = a.Xexp + (long long)g * a.k;
        } else if (g < leaf_groups) {
          erow = a.Dexp[i];
          ecol = a.Xexp + ((lrow0 + g * 64) / kOzChunk) * a.k;
        } else {
          const int l = g - leaf_groups;
          erow = a.Uexp[(long long)l * a.n + i];
          ecol = a.Texp + a.lteo[l] + (it.row0 / a.lrows[l]) * a.k;
        }
        ec = jl < a.k ? __ldg(ecol + jl) : 0;
      };
      auto next_group = [&](int g) {
        do ++g;
        while (g < it.g1 && !group_exists<MODE>(a, it, g));
        return g;
      };
      float rh[kEpiCols], rl[kEpiCols];
#pragma unroll
      for (int c = 0; c < kEpiCols; ++c) rh[c] = rl[c] = 0.f;
      int erow_n, ec_n;
      exps(it.g0, erow_n, ec_n);
      for (int g = it.g0; ok && g < it.g1; g = next_group(g)) {
        const unsigned par = (unsigned)(gcount & 1);
        ++gcount;
        const int er = erow_n - 14, ec = ec_n;
        const int gn = next_group(g);
        if (gn < it.g1) exps(gn, erow_n, ec_n);
        const bool fast = __all_sync(0xffffffffu, er + __reduce_max_sync(0xffffffffu, ec) <= 127 &&
                                                      er + __reduce_min_sync(0xffffffffu, ec) - 42 >= -126);
        // region 0: diagonals 0-3; region 1: diagonals 4-6
        if (!wait_or_abort(&sh->acc_full[0], par, sh)) {
          ok = false;
          break;
        }
        tc_fence_after();
        if (!idle) drain_region<4, 0>(tl, rh, rl, er, ec, fast);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) arrive(&sh->acc_empty[0]);
        if (!wait_or_abort(&sh->acc_full[1], par, sh)) {
          ok = false;
          break;
        }
        tc_fence_after();
        if (!idle) drain_region<3, 4>(tl + (unsigned)(4 * kCols), rh, rl, er, ec, fast);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) arrive(&sh->acc_empty[1]);
        if constexpr (MODE == 1) {
          if (valid && rows1 <= a.R) {
            // a block of this level ends with this chunk: its T is complete
            const long long end = (long long)(g + 1) * 64;
            if ((end & (rows1 - 1)) == 0) {
              const long long b = end / rows1 - 1;
              if (b < a.lnb[l1]) store_fp64(a.T + a.toff[l1] + b * a.r * a.k + qq, a.r, rh, rl, jb, a.k);
#pragma unroll
              for (int c = 0; c < kEpiCols; ++c) rh[c] = rl[c] = 0.f;
            }
          }
        }
      }
      if (!ok) break;
      if constexpr (MODE == 1) {
        if (valid && rows1 > a.R) {  // this range's part of a longer block
          const long long b = it.row0 / rows1, part = (it.row0 & (rows1 - 1)) / a.R;
          if (b < a.lnb[l1])
            store_fp64(a.P + a.poff[l1] + (b * a.parts[l1] + part) * a.r * a.k + qq, a.r, rh, rl, jb, a.k);
        }
      } else {
#pragma unroll
        for (int c = 0; c < kEpiCols; ++c) {
          const int j = jb + c;
          if (j >= a.k) continue;
          const float2 bv = split_bits(a.B[i + (long long)j * a.ldb]);
          float s, e;
          two_sum(bv.x, -rh[c], s, e);
          e += bv.y - rl[c];
          const float h = s + e;
          a.R2[i + (long long)j * a.ldr] = make_float2(h, e - (h - s));
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && sh->abort) report_error(a.st, HODLR_ERR_TIMEOUT, blockIdx.x);
  if (threadIdx.x == 0 && sh->abort) {
    // copies the producer issued but nobody consumed: wait (bounded) for them to land
    for (long long it = sh->consumed; it < issued; ++it) {
      const long long t0 = clock64();
      while (!mbar_try_wait(&sh->full[it % kStages], (unsigned)((it / kStages) & 1)) && clock64() - t0 < kWaitCycles) {
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tc_dealloc(tmem, kTmemCols);
  }
}

// The partial sums of every level with blocks longer than a range, in one
// launch: thread e of level slot i (e < nb r k) sums its element's parts in
// a fixed order (four interleaved accumulators, combined pairwise).
struct Pass2Levels {
  long long pre[kMaxLevels + 1], toff[kMaxLevels], poff[kMaxLevels];
  int parts[kMaxLevels], n;
  long long blk;
};
__global__ void oz_tc_pass2_kernel(const double *__restrict__ P, double *T, Pass2Levels a, const int *skip) {
  if (skip && *skip) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.pre[a.n]) return;
  int i = 0;
  while (e >= a.pre[i + 1]) ++i;
  const long long le = e - a.pre[i], b = le / a.blk, x = le % a.blk;
  const int parts = a.parts[i];
  const double *p = P + a.poff[i] + b * parts * a.blk + x;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int c = 0;
  for (; c + 4 <= parts; c += 4) {
    s0 += p[(long long)c * a.blk];
    s1 += p[(long long)(c + 1) * a.blk];
    s2 += p[(long long)(c + 2) * a.blk];
    s3 += p[(long long)(c + 3) * a.blk];
  }
  for (; c < parts; ++c) s0 += p[(long long)c * a.blk];
  T[a.toff[i] + b * a.blk + x] = (s0 + s1) + (s2 + s3);
}

static bool is_pow2(long long v) { return v > 0 && (v & (v - 1)) == 0; }

static cudaError_t launch_mode(int mode, const CUtensorMap &a0, const CUtensorMap &b0, const CUtensorMap &a1,
                               const CUtensorMap &b1, const OzTcArgs &a, cudaStream_t s) {
  const size_t bytes = (size_t)kStages * kStageBytes + sizeof(Shared) + 1024;
  auto kern = mode == 0 ? oz_tc_kernel<0> : oz_tc_kernel<1>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  const long long grid = persistent_ctas(a.items);
  HODLR_LAUNCH(kern, (unsigned)grid, kThreads, bytes, s, a0, b0, a1, b1, a);
  return cudaGetLastError();
}

bool oz_tc_supported(int m, int r, int k) {
  return (m == 128 || m == 256) && r % 8 == 0 && r >= 8 && r <= 64 && k >= 1;
}

cudaError_t launch_oz_tc_resid(const __nv_bfloat16 *Dsl, const int *Dexp, const __nv_bfloat16 *Xsl, const int *Xexp,
                               const __nv_bfloat16 *Usl, const int *Uexp, const __nv_bfloat16 *Tsl, const int *Texp,
                               long long n, int m, int L, int r, int k, const int *lev_nb, const long long *lev_rows,
                               const double *B, long long ldb, float2 *R2, long long ldr, const int *skip,
                               DevStatus *st, cudaStream_t s) {
  if (k <= 0 || n <= 0) return cudaSuccess;
  if (!oz_tc_supported(m, r, k) || n % kRows || L > kMaxLevels) return cudaErrorInvalidValue;
  OzTcArgs a{};
  long long nt_rows = 0, neo = 0;
  for (int l = 0; l < L; ++l) {
    if (lev_rows[l] % kRows) return cudaErrorInvalidValue;
    a.lrows[l] = lev_rows[l];
    a.lnb[l] = lev_nb[l];
    a.ltrow[l] = nt_rows;
    a.lteo[l] = neo;
    nt_rows += (long long)lev_nb[l] * kOzSlices * k;
    neo += (long long)lev_nb[l] * k;
  }
  CUtensorMap mD, mX, mU, mT;
  if (!make_tensor_map_bf16(&mD, Dsl, m, (long long)kOzSlices * n, m, kSlab, kRows, 64) ||
      !make_tensor_map_bf16(&mX, Xsl, n, (long long)kOzSlices * k, n, kSlab, kCols, 64) ||
      !make_tensor_map_bf16(&mU, L > 0 ? (const void *)Usl : (const void *)Dsl, L > 0 ? r : m,
                            L > 0 ? (long long)kOzSlices * L * n : 1, L > 0 ? r : m, kSlab, kRows, 64) ||
      !make_tensor_map_bf16(&mT, L > 0 ? (const void *)Tsl : (const void *)Dsl, L > 0 ? r : m,
                            L > 0 ? nt_rows : 1, L > 0 ? r : m, kSlab, kCols, 64))
    return cudaErrorInvalidValue;
  a.Dexp = Dexp;
  a.Xexp = Xexp;
  a.Uexp = Uexp;
  a.Texp = Texp;
  a.B = B;
  a.ldb = ldb;
  a.R2 = R2;
  a.ldr = ldr;
  a.n = n;
  a.m = m;
  a.L = L;
  a.r = r;
  a.k = k;
  a.nct = (k + kCols - 1) / kCols;
  a.items = (n / kRows) * a.nct;
  a.skip = skip;
  a.st = st;
  return launch_mode(0, mD, mX, mU, mT, a, s);
}

// Rows per reduction range: the largest power of two <= 2048 dividing n.
static long long reduce_range(long long n) {
  long long R = 2048;
  while (R > kRows && n % R) R >>= 1;
  return R;
}

size_t oz_tc_reduce_partials(long long n, int L, int r, int k, const int *lev_nb, const long long *lev_rows) {
  const long long R = reduce_range(n);
  size_t tot = 0;
  for (int l = 0; l < L; ++l)
    if (lev_rows[l] > R) tot += (size_t)lev_nb[l] * (size_t)(lev_rows[l] / R) * r * k;
  return tot;
}

cudaError_t launch_oz_tc_reduce(const __nv_bfloat16 *Vsl, const int *Vexp, const __nv_bfloat16 *Xsl,
                                const int *Xexp, long long n, int L, int r, int k, const int *lev_nb,
                                const long long *lev_rows, double *T, double *P, const int *skip, DevStatus *st,
                                cudaStream_t s) {
  if (k <= 0 || n <= 0 || L <= 0) return cudaSuccess;
  if (r % 8 || r < 8 || r > 64 || n % kRows || L > kMaxLevels) return cudaErrorInvalidValue;
  OzTcArgs a{};
  a.R = reduce_range(n);
  long long toff = 0, poff = 0;
  for (int l = 0; l < L; ++l) {
    if (!is_pow2(lev_rows[l]) || lev_rows[l] % kOzChunk) return cudaErrorInvalidValue;
    a.lrows[l] = lev_rows[l];
    a.lnb[l] = lev_nb[l];
    a.toff[l] = toff;
    toff += (long long)lev_nb[l] * r * k;
    a.parts[l] = lev_rows[l] > a.R ? (int)(lev_rows[l] / a.R) : 0;
    a.poff[l] = poff;
    poff += (long long)lev_nb[l] * a.parts[l] * r * k;
  }
  CUtensorMap mV, mX;
  if (!make_tensor_map_bf16(&mV, Vsl, n, (long long)kOzSlices * L * r, n, kSlab, kRows, 64) ||
      !make_tensor_map_bf16(&mX, Xsl, n, (long long)kOzSlices * k, n, kSlab, kCols, 64))
    return cudaErrorInvalidValue;
  a.Vexp = Vexp;
  a.Xexp = Xexp;
  a.T = T;
  a.P = P;
  a.n = n;
  a.m = 128;
  a.L = L;
  a.r = r;
  a.k = k;
  a.QL = kRows / r;
  a.nstack = (L + a.QL - 1) / a.QL;
  a.nct = (k + kCols - 1) / kCols;
  a.items = ((n + a.R - 1) / a.R) * a.nstack * a.nct;
  a.skip = skip;
  a.st = st;
  cudaError_t e = launch_mode(1, mV, mX, mV, mX, a, s);
  if (e != cudaSuccess) return e;
  Pass2Levels p2{};
  p2.blk = (long long)r * k;
  long long pre = 0;
  for (int l = 0; l < L; ++l)
    if (a.parts[l] > 0) {
      p2.pre[p2.n] = pre;
      p2.toff[p2.n] = a.toff[l];
      p2.poff[p2.n] = a.poff[l];
      p2.parts[p2.n] = a.parts[l];
      pre += (long long)lev_nb[l] * p2.blk;
      ++p2.n;
    }
  p2.pre[p2.n] = pre;
  if (pre > 0) HODLR_LAUNCH(oz_tc_pass2_kernel, (unsigned)ceil_div(pre, 256), 256, 0, s, P, T, p2, skip);
  return cudaGetLastError();
}

}  // namespace hodlr
