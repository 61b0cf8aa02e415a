// D^{-1} U for 128-row leaves on the tcgen05 tensor cores: the mixed
// factorisation's first leaf application, Utilde(leaf rows, :) = Dinv_leaf
// U(leaf rows, :) over all L r columns of U at once, U read in FP64 (rounded
// to FP32 as it is split) and Utilde written in FP32 -- the leaf solve of
// hsolve (src/tasks/leaf_solve.cc:87-92, dgesv on the d0/d1 blocks against
// every column of u) applied through the explicit FP32 inverse.
//
// Both operands are cut into exact bf16 planes (x = h + m + l, as in the
// low-rank update), and the six partial products down to 2^-16 come from
// three N-concatenated products per K-step,
//   A_h [B_h B_m B_l]  ->  accumulator columns  0 .. 95
//   A_m [B_h B_m]      ->                       32 .. 95
//   A_l [B_h]          ->                       64 .. 95,
// so that the three 32-column groups hold hh | hm + mh | hl + mm + lh; the
// epilogue sums them smallest first.  FP32-class accurate (the three dropped
// products are below 2^-23 of |a b| together), the class of the FMA kernel
// this replaces.
//
// A = Dinv lives in tensor memory: its three planes (128 lanes x 64 columns
// each, two bf16 a column) are cut once per leaf and serve all of the leaf's
// ceil(L r / 32) tiles, so the products read only the 24 KB of U planes from
// shared memory -- shared-memory bandwidth, not the tensor cores, bounds a
// kernel that re-reads a 96 KB operand for every 32 output columns.  One
// persistent CTA per SM walks a contiguous range of (leaf, 32-column) tiles;
// the producer prefetches the next leaf's Dinv into L2 when a leaf starts.
// The U tiles stream through a 4-stage TMA ring and the U planes are
// double-buffered, so that the split of tile i + 1 runs while the tensor
// cores multiply tile i.  Warp roles, joined by mbarriers: 16 splitters,
// 8 epilogue warps (tensor memory -> registers -> global, one row and 16
// columns a thread, coalesced along the rows), a producer and an MMA issuer.
// The splits are chains of dependent conversions, so it takes many warps to
// keep them from pacing the tiles.  Every wait is bounded; on timeout the
// CTA records HODLR_ERR_TIMEOUT, waits (bounded) for its copies and products
// and frees its tensor memory.
#include <cuda_bf16.h>

#include <cstdlib>

#include "kernels.cuh"
#include "tcgen05.cuh"
#include "tma.cuh"

namespace hodlr {

namespace {

constexpr int kLM = 128;                       // leaf rows = K of the product
constexpr int kLBN = 32;                       // columns of U per tile
constexpr int kLStages = 4;                    // U tiles in flight
constexpr int kLStageBytes = kLM * kLBN * 8;   // one FP64 U tile: 32 KB
constexpr int kLPlaneB = kLBN * 64;            // 32 K values of one U plane's 32 rows: 2 KB
constexpr int kLChunkB = 3 * kLPlaneB;         // the three U planes of one K chunk (96 rows)
constexpr int kLSW = 16;                       // splitter warps
constexpr int kLEW = 8;                        // epilogue warps: 4 lane quarters x 2 column halves
constexpr int kLThreads = 32 * (kLSW + kLEW + 2);  // + producer, MMA
constexpr int kLSplit = 32 * kLSW;
constexpr int kLBufB = 4 * kLChunkB;           // one buffer of U planes: 24 KB
constexpr size_t kLSmem = (size_t)kLStages * kLStageBytes + 2 * kLBufB + 1024;
// tensor-memory columns: accumulators at 0 and 128 (96 each), the Dinv
// planes at 256, 320, 384 (64 each: 128 K values, two a column)
constexpr unsigned kLTmemCols = 512, kLAcc = 128, kLTA = 256, kLTPlane = 64;
constexpr long long kLWait = 2000000000LL;     // about one second of SM clocks

struct LaShared {
  uint64_t full[kLStages], stage_free[kLStages];
  uint64_t planes_ready[2], planes_free[2], acc_full[2], acc_free[2], drain;
  unsigned tmem;
  int abort;
};

__device__ __forceinline__ void prefetch_l2(const void *p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

}  // namespace

__global__ void __launch_bounds__(kLThreads, 1)
leaf_apply_tc_kernel(const __grid_constant__ CUtensorMap mapX, const float *__restrict__ Dinv, float *Y,
                     long long ldy, int ncols, int nct, int nleaf, DevStatus *st) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char *pb = base + kLStages * kLStageBytes;  // 2 buffers of 4 K chunks of the 3 U planes' 96 rows
  __shared__ LaShared shm;
  LaShared *sh = &shm;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long ntiles = (long long)nleaf * nct;
  const long long t0 = ntiles * blockIdx.x / gridDim.x, t1 = ntiles * (blockIdx.x + 1) / gridDim.x;
  const long long nmine = t1 - t0;
  if (tid == 0) {
    prefetch_tensormap(&mapX);
    for (int q = 0; q < kLStages; ++q) {
      mbar_init(&sh->full[q], 1);
      mbar_init(&sh->stage_free[q], kLSplit);
    }
    for (int q = 0; q < 2; ++q) {
      mbar_init(&sh->planes_ready[q], kLSplit);
      mbar_init(&sh->planes_free[q], 1);
      mbar_init(&sh->acc_full[q], 1);
      mbar_init(&sh->acc_free[q], 32 * kLEW);
    }
    mbar_init(&sh->drain, 1);
    sh->abort = 0;
    mbar_fence_init();
  }
  constexpr int kProd = kLSW + kLEW, kMmaWarp = kProd + 1;
  static_assert(kLSW == 16 && kLBN * 16 == 32 * kLSW, "warp roles: 4 quarters x 4 K ranges; one U task a thread");
  if (warp == kMmaWarp) {
    tc_alloc(&sh->tmem, kLTmemCols);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = sh->tmem;
  auto wait = [&](uint64_t *bar, unsigned parity) { return mbar_wait_or_abort(bar, parity, &sh->abort, kLWait); };
  long long issued = 0;  // tiles whose loads were issued (producer)
  if (warp == kProd) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      for (long long j = 0; j < nmine; ++j) {
        const int s = (int)(j % kLStages);
        if (j >= kLStages && !wait(&sh->stage_free[s], (unsigned)((j / kLStages - 1) & 1))) break;
        const long long t = t0 + j;
        const int leaf = (int)(t / nct), ct = (int)(t - (long long)leaf * nct);
        if (j == 0) prefetch_l2(Dinv + (long long)leaf * kLM * kLM, kLM * kLM * 4);
        if ((j == 0 || ct == 0) && leaf + 1 < nleaf)
          prefetch_l2(Dinv + (long long)(leaf + 1) * kLM * kLM, kLM * kLM * 4);
        mbar_arrive_expect_tx(&sh->full[s], kLStageBytes);
        tma_load_2d(base + s * kLStageBytes, &mapX, &sh->full[s], leaf * kLM, ct * kLBN);
        issued = j + 1;
      }
    }
  } else if (warp == kMmaWarp) {
    // ---------------------------------------------------------------- MMA
    if (lane == 0) {
      const unsigned id96 = tc_idesc_bf16(kLM, 96), id64 = tc_idesc_bf16(kLM, 64), id32 = tc_idesc_bf16(kLM, 32);
      const unsigned b0 = smem_u32(pb);
      for (long long i = 0; i < nmine; ++i) {
        const int ac = (int)(i & 1);  // the accumulator and the plane buffer of tile i
        if (!wait(&sh->planes_ready[ac], (unsigned)((i >> 1) & 1))) break;
        if (i >= 2 && !wait(&sh->acc_free[ac], (unsigned)(((i >> 1) - 1) & 1))) break;
        tc_fence_after();
        const unsigned d = tmem + kLAcc * ac, ta = tmem + kLTA;
        // B descriptors as base + offset (16-byte units; every shared address
        // fits the 14-bit field), the base opaque so that the eight are formed
        // per tile instead of held in registers
        uint64_t db = desc_sw64(b0 + ac * kLBufB);
        asm volatile("" : "+l"(db));
#pragma unroll
        for (int ks = 0; ks < 8; ++ks) {  // K steps of 16: chunk ks / 2, half ks % 2
          const uint64_t bd = db + ((ks >> 1) * kLChunkB >> 4) + 2 * (ks & 1);
          tc_mma_ta(d, ta + 8 * ks, bd, id96, ks ? 1u : 0u);
          tc_mma_ta(d + 32, ta + kLTPlane + 8 * ks, bd, id64, 1u);
          tc_mma_ta(d + 64, ta + 2 * kLTPlane + 8 * ks, bd, id32, 1u);
        }
        tc_commit(&sh->acc_full[ac]);
        tc_commit(&sh->planes_free[ac]);
      }
      tc_commit(&sh->drain);  // completes once every product issued above has
      const long long c0 = clock64();
      while (!mbar_try_wait(&sh->drain, 0) && clock64() - c0 < kLWait) {
      }
    }
  } else if (warp < kLSW) {
    // ----------------------------------------------------------- splitters
    int cur = -1;
    for (long long i = 0; i < nmine; ++i) {
      const int s = (int)(i % kLStages);
      const long long t = t0 + i;
      const int leaf = (int)(t / nct);
      if (!wait(&sh->full[s], (unsigned)((i / kLStages) & 1))) break;
      const int pbuf = (int)(i & 1);
      // the products of tile i - 2 have read this plane buffer; before the
      // Dinv planes change, those of tile i - 1 have read them too
      if (i >= 2 && !wait(&sh->planes_free[pbuf], (unsigned)(((i >> 1) - 1) & 1))) break;
      if (leaf != cur && i >= 1 && !wait(&sh->planes_free[pbuf ^ 1], (unsigned)(((i - 1) >> 1) & 1))) break;
      if (leaf != cur) {
        // Dinv planes into tensor memory: warp w writes lanes 32 q .. 32 q + 31
        // (q = w mod 4, the quarter its index allows) and K values 32 g ..
        // 32 g + 31 (g = w / 4); the loads are coalesced along the rows, two
        // tasks of 8 K values in flight at a time
        const float *A = Dinv + (long long)leaf * kLM * kLM;
        const int q = warp & 3, g = warp >> 2, r = 32 * q + lane;
        const unsigned tl = tmem + ((unsigned)(32 * q) << 16) + kLTA;
#pragma unroll
        for (int u0 = 0; u0 < 4; u0 += 2) {
          float x[2][8];
#pragma unroll
          for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int e = 0; e < 8; ++e) x[u][e] = __ldg(A + (long long)(32 * g + 8 * (u0 + u) + e) * kLM + r);
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            uint4 h, m, l;
            split3_pair(x[u][0], x[u][1], h.x, m.x, l.x);
            split3_pair(x[u][2], x[u][3], h.y, m.y, l.y);
            split3_pair(x[u][4], x[u][5], h.z, m.z, l.z);
            split3_pair(x[u][6], x[u][7], h.w, m.w, l.w);
            const unsigned col = (32 * g + 8 * (u0 + u)) / 2;
            tc_st4(tl + col, h);
            tc_st4(tl + kLTPlane + col, m);
            tc_st4(tl + 2 * kLTPlane + col, l);
          }
        }
        tc_wait_st();
        cur = leaf;
      }
      // U planes: task (column j, 8 K values c), FP64 -> FP32 (on the
      // integer pipes) -> 3 x bf16.  The eight lanes of a shared-memory
      // phase take columns j0, j0 + 1 and four chunks of one 32-value K
      // range, and start their four 16-byte reads at distinct offsets: the
      // reads and the swizzled plane writes are free of bank conflicts.
      const double *sX = reinterpret_cast<const double *>(base + s * kLStageBytes);  // [kLBN][kLM]
#pragma unroll
      for (int u = 0; u < kLBN * 16 / kLSplit; ++u) {
        const int t = tid + kLSplit * u, kc = (t >> 3) & 3;
        const int j = ((t >> 5) << 1) | ((t >> 2) & 1), c = 4 * kc + (t & 3);
        const int d = (((c >> 1) & 1) + 2 * (j & 1)) & 3;  // the first 16-byte piece read
        double2 w[4];
#pragma unroll
        for (int e2 = 0; e2 < 4; ++e2)
          w[e2] = *reinterpret_cast<const double2 *>(sX + j * kLM + 8 * c + 2 * ((e2 + d) & 3));
        float x[8];
#pragma unroll
        for (int p2 = 0; p2 < 4; ++p2) {  // piece p2 sits in w[(p2 - d) & 3]
          const double2 v = d == 0 ? w[p2] : d == 1 ? w[(p2 + 3) & 3] : d == 2 ? w[(p2 + 2) & 3] : w[(p2 + 1) & 3];
          x[2 * p2] = f64_to_f32_rn(v.x);
          x[2 * p2 + 1] = f64_to_f32_rn(v.y);
        }
        put_planes(pb + pbuf * kLBufB + kc * kLChunkB, kLPlaneB, swz64(j, c & 3), x);
      }
      tc_fence_before();  // the tensor-memory writes above, before the arrival the MMA thread waits on
      mbar_arrive(&sh->stage_free[s]);
      fence_proxy_async_smem();  // the planes are read by the tensor core (async proxy)
      mbar_arrive(&sh->planes_ready[pbuf]);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    // warp w reads tensor-memory lanes 32 q .. 32 q + 31 (q = w mod 4, the
    // quarter its warp index allows) and the columns of half hh of each group
    const int q = warp & 3, hh = (warp - kLSW) >> 2, r = 32 * q + lane;
    for (long long i = 0; i < nmine; ++i) {
      const int ac = (int)(i & 1);
      // warp-uniform outcome: tcgen05.ld below is a warp-collective instruction
      if (!__all_sync(0xffffffffu, wait(&sh->acc_full[ac], (unsigned)((i >> 1) & 1)))) break;
      tc_fence_after();
      // the two smaller groups first (32 registers), then the leading one
      const unsigned tl = tmem + ((unsigned)(32 * q) << 16) + (unsigned)(128 * ac + 16 * hh);
      unsigned v[2][16];
      tc_ld16(tl + 64, v[0]);
      tc_ld16(tl + 32, v[1]);
      tc_wait_ld(v);
      float o[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) o[j] = __uint_as_float(v[0][j]) + __uint_as_float(v[1][j]);
      tc_ld16(tl, v[0]);
      tc_wait_ld(v);
      tc_fence_before();
      mbar_arrive(&sh->acc_free[ac]);
#pragma unroll
      for (int j = 0; j < 16; ++j) o[j] += __uint_as_float(v[0][j]);
      const long long t = t0 + i;
      const int leaf = (int)(t / nct), ct = (int)(t - (long long)leaf * nct), c0 = ct * kLBN;
      const int nc = min(kLBN, ncols - c0) - 16 * hh;
      float *y = Y + (long long)leaf * kLM + r + (long long)(c0 + 16 * hh) * ldy;
#pragma unroll
      for (int j = 0; j < 16; ++j, y += ldy)
        if (j < nc) *y = o[j];
    }
  }
  __syncthreads();
  if (tid == 32 * kProd && sh->abort) {  // the producer thread
    report_error(st, HODLR_ERR_TIMEOUT, blockIdx.x);
    // loads issued but possibly still landing: wait (bounded) for them
    for (long long j = issued > kLStages ? issued - kLStages : 0; j < issued; ++j) {
      const long long c0 = clock64();
      while (!mbar_try_wait(&sh->full[j % kLStages], (unsigned)((j / kLStages) & 1)) && clock64() - c0 < kLWait) {
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    tc_dealloc(tmem, kLTmemCols);
  }
}

// Utilde = Dinv U on the tensor cores for 128-row leaves, U in FP64 (column-
// major, ld lds), Utilde in FP32 (ld ldy).  False if the preconditions do
// not hold (the caller takes the FMA kernel).
bool leaf_apply_tc_try(const float *Dinv, int nleaf, const double *U, long long lds, float *Y, long long ldy,
                       int ncols, DevStatus *st, cudaStream_t s, cudaError_t &err) {
  err = cudaSuccess;
  const char *off = getenv("HODLR_NO_TCGEN05");
  if ((off && off[0] == '1') || current_tuning().leaf_apply == 1) return false;
  if (nleaf < 1 || ncols < 1 || (reinterpret_cast<uintptr_t>(Dinv) & 15)) return false;
  CUtensorMap mx;
  if (!make_tensor_map_f64(&mx, U, (long long)nleaf * kLM, ncols, lds, kLM, kLBN)) return false;
  err = allow_dyn_smem(leaf_apply_tc_kernel, kLSmem);
  if (err != cudaSuccess) return true;
  const int nct = (ncols + kLBN - 1) / kLBN;
  const long long grid = persistent_ctas((long long)nleaf * nct);
  HODLR_LAUNCH(leaf_apply_tc_kernel, (unsigned)grid, kLThreads, kLSmem, s, mx, Dinv, Y, ldy, ncols, nct, nleaf, st);
  err = cudaGetLastError();
  return true;
}

}  // namespace hodlr
