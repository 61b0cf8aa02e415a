// K3 on the tcgen05 tensor cores: the row reductions Out_b = V_b^T X_b of the
// mixed path (FP32 operands, rank <= 32), FP32-class accurate.
//
// The reference forms these blocks with dgemm('t', 'n') inside hsolve
// (src/tasks/leaf_solve.cc:132-135) and GemmRedTask (src/tasks/
// gemm_reduce.cc:33-83).  Here a block product is D = X^T V (M = 128 columns
// of X, N = the ranks, K = the rows), every FP32 operand cut exactly into
// three bf16 planes (x = h + m + l, as the tensor-core update does) and the
// six products down to 2^-16 issued as tcgen05.mma into tensor-memory
// accumulators.  An accumulator is used for 128 rows at a time only: four
// epilogue warps then move it into FP32 registers with round-to-nearest adds
// (tcgen05.ld), so a sum over a long row chunk is a sum of short exact-input
// partial products in FP32 -- not one accumulator running over thousands of
// rows, whose accumulation rounding showed in the refined residual.
//
// One persistent CTA per SM walks work units (child block b, row chunk,
// 128-column tile of X) with warp roles joined by mbarriers:
// * one thread issues the TMA loads of 64-row stages (X: 64 rows x 128
//   columns = 32 KB, V: 64 rows x 32 ranks, FP32) into a 3-deep ring, as 3-D
//   boxes of two 32-row blocks so that the 128-byte swizzle applies (boxes
//   of 16 KB streamed at no more than ~4.7 TB/s on this GPU, of 32 KB at
//   ~7.4 TB/s);
// * sixteen warps cut each stage, one 32-row half at a time, into planes
//   (K-major, 64-byte swizzle, double buffered per half; 8 lanes read one
//   128-byte line, so the reads are free of bank conflicts; one mbarrier
//   arrival per warp);
// * one thread issues a half's products: V's three planes are stacked along
//   N, so h x [Vh|Vm|Vl] (N 96), m x [Vh|Vm] (N 64) and l x Vh (N 32) are the
//   six products in three instructions per K-step of 16, landing in three
//   32-column blocks of one of two accumulators;
// * four warps drain an accumulator every 128 rows, adding its three blocks
//   into the FP32 sums, and write each unit's r x 128 partial block
//   (split-K partials are summed by the fixed-order second pass).
// Every wait is bounded; on a timeout every role stops, in-flight copies and
// products are waited for (bounded), the tensor memory is released and
// HODLR_ERR_TIMEOUT recorded.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>

#include "kernels.cuh"
#include "tcgen05.cuh"
#include "tma.cuh"

namespace hodlr {

// Test hook of the bounded waits (struct WaitFault), this kernel's copy.
__device__ WaitFault g_rc_wait_fault = {-1, -1, 0};

cudaError_t reduce_tc_set_wait_fault(const WaitFault &wf) {
  return cudaMemcpyToSymbol(g_rc_wait_fault, &wf, sizeof wf);
}

namespace {

constexpr int kRcM = 128, kRcN = 32;              // X columns per unit, ranks (one accumulator block)
constexpr int kRcK = 64, kRcH = 32;               // rows per stage, rows per half (planes)
constexpr int kRcStages = 3, kRcGroup = 4;        // ring depth; halves per accumulator use (128 rows)
constexpr int kRcAcc = 3 * kRcN;                  // columns of one accumulator
constexpr int kRcTmemCols = 256;                  // two accumulators, rounded up to a power of two
constexpr int kRcSplitWarps = 16, kRcThreads = 32 * (kRcSplitWarps + 6);
constexpr int kRcXBytes = kRcK * kRcM * 4;        // FP32 X stage: 32 KB
constexpr int kRcVBytes = kRcK * kRcN * 4;        // FP32 V stage: 8 KB
constexpr int kRcStageBytes = kRcXBytes + kRcVBytes;
constexpr int kRcPX = kRcM * kRcH * 2;            // one bf16 plane of half an X stage: 8 KB
constexpr int kRcPV = kRcN * kRcH * 2;            // one bf16 plane of half a V stage: 2 KB
constexpr int kRcPlaneSet = 3 * kRcPX + 3 * kRcPV;
constexpr size_t kRcSmem = (size_t)kRcStages * kRcStageBytes + 2 * (size_t)kRcPlaneSet + 1024;
constexpr long long kRcWait = 2000000000LL;       // about one second of SM clocks

struct RcShared {
  uint64_t full[kRcStages], slot_free[kRcStages];
  uint64_t planes_ready[2], planes_free[2], acc_full[2], acc_free[2], drain;
  long long budget;
  unsigned tmem;
  int abort;
};

__device__ __forceinline__ bool rc_wait(uint64_t *bar, unsigned parity, RcShared *sh) {
  return mbar_wait_or_abort(bar, parity, &sh->abort, sh->budget);
}

struct RcArgs {
  long long nrows;  // rows per child block
  int nbatch, r, C, chunk_rows, nchunks, nct;
  long long nunits;
  const int *skip;
  DevStatus *st;
};

}  // namespace

template <typename OutT>
__global__ void __launch_bounds__(kRcThreads, 1)
reduce_tc_kernel(const __grid_constant__ CUtensorMap mapX, const __grid_constant__ CUtensorMap mapV, RcArgs a,
                 OutT *out) {
  if (a.skip && *a.skip) return;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char *planes = base + kRcStages * kRcStageBytes;  // 2 sets of (3 X planes, 3 V planes) of a half
  __shared__ RcShared shm;
  RcShared *sh = &shm;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int kEpi0 = kRcSplitWarps, kProd = kRcSplitWarps + 4, kMma = kRcSplitWarps + 5;
  constexpr int kSplitThreads = 32 * kRcSplitWarps;
  const WaitFault wf = g_rc_wait_fault;
  const long long skip_stage = wf.cta == (int)blockIdx.x ? wf.stage : -1;

  // unit i of this CTA -> (column tile, chunk, block), its first row and stage count
  auto unit = [&](long long i, int &ct, int &chunk, int &b, int &row0, int &nst) {
    long long lin = blockIdx.x + i * gridDim.x;
    ct = (int)(lin % a.nct);
    lin /= a.nct;
    chunk = (int)(lin % a.nchunks);
    b = (int)(lin / a.nchunks);
    row0 = (int)((long long)b * a.nrows + (long long)chunk * a.chunk_rows);
    const long long rows = std::min<long long>(a.chunk_rows, a.nrows - (long long)chunk * a.chunk_rows);
    nst = (int)(rows / kRcK);
  };
  const long long nmine = a.nunits > blockIdx.x ? (a.nunits - 1 - blockIdx.x) / gridDim.x + 1 : 0;

  if (tid == 0) {
    prefetch_tensormap(&mapX);
    prefetch_tensormap(&mapV);
    for (int q = 0; q < kRcStages; ++q) {
      mbar_init(&sh->full[q], 1);
      mbar_init(&sh->slot_free[q], kRcSplitWarps);
    }
    for (int q = 0; q < 2; ++q) {
      mbar_init(&sh->planes_ready[q], kRcSplitWarps);
      mbar_init(&sh->planes_free[q], 1);
      mbar_init(&sh->acc_full[q], 1);
      mbar_init(&sh->acc_free[q], 4);
    }
    mbar_init(&sh->drain, 1);
    sh->budget = skip_stage >= 0 && wf.budget > 0 ? wf.budget : kRcWait;
    sh->abort = 0;
    mbar_fence_init();
  }
  if (warp == kMma) {
    tc_alloc(&sh->tmem, kRcTmemCols);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = sh->tmem;
  long long issued = 0;  // stages whose loads were issued (producer)

  if (warp == kProd) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      long long g = 0;
      for (long long i = 0; i < nmine && !sh->abort; ++i) {
        int ct, chunk, b, row0, nst;
        unit(i, ct, chunk, b, row0, nst);
        for (int s = 0; s < nst; ++s, ++g) {
          const int q = (int)(g % kRcStages);
          if (g >= kRcStages && !rc_wait(&sh->slot_free[q], (unsigned)(((g / kRcStages) - 1) & 1), sh)) break;
          if (g != skip_stage) {
            unsigned char *sx = base + q * kRcStageBytes;
            const int blk = (row0 + s * kRcK) / 32;  // first 32-row block of the stage
            mbar_arrive_expect_tx(&sh->full[q], kRcStageBytes);
            tma_load_3d(sx, &mapX, &sh->full[q], 0, blk, ct * kRcM);
            tma_load_3d(sx + kRcXBytes, &mapV, &sh->full[q], 0, blk, 0);
          }
          issued = g + 1;
        }
      }
    }
  } else if (warp == kMma) {
    // ---------------------------------------------------------------- MMA
    if (lane == 0) {
      const unsigned id96 = tc_idesc_bf16(kRcM, 3 * kRcN), id64 = tc_idesc_bf16(kRcM, 2 * kRcN),
                     id32 = tc_idesc_bf16(kRcM, kRcN);
      long long gh = 0, grp = 0;  // halves processed, accumulator uses
      for (long long i = 0; i < nmine && !sh->abort; ++i) {
        int ct, chunk, b, row0, nst;
        unit(i, ct, chunk, b, row0, nst);
        const int nh = 2 * nst;
        bool ok = true;
        for (int hs = 0; hs < nh; ++hs, ++gh) {
          const int pb = (int)(gh & 1), ac = (int)(grp & 1);
          const bool first = hs % kRcGroup == 0, last = hs % kRcGroup == kRcGroup - 1 || hs == nh - 1;
          if (!rc_wait(&sh->planes_ready[pb], (unsigned)((gh >> 1) & 1), sh)) {
            ok = false;
            break;
          }
          if (first && grp >= 2 && !rc_wait(&sh->acc_free[ac], (unsigned)(((grp >> 1) - 1) & 1), sh)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const unsigned d = tmem + (unsigned)(kRcAcc * ac);
          unsigned char *px = planes + pb * kRcPlaneSet, *pv = px + 3 * kRcPX;
          const uint64_t bv = desc_sw64(smem_u32(pv));  // [Vh | Vm | Vl] stacked along N
#pragma unroll
          for (int kk = 0; kk < kRcH / 16; ++kk) {
            tc_mma(d, desc_sw64(smem_u32(px)) + 2 * kk, bv + 2 * kk, id96, (first && kk == 0) ? 0u : 1u);
            tc_mma(d, desc_sw64(smem_u32(px + kRcPX)) + 2 * kk, bv + 2 * kk, id64, 1u);
            tc_mma(d, desc_sw64(smem_u32(px + 2 * kRcPX)) + 2 * kk, bv + 2 * kk, id32, 1u);
          }
          tc_commit(&sh->planes_free[pb]);
          if (last) {
            tc_commit(&sh->acc_full[ac]);
            ++grp;
          }
        }
        if (!ok) break;
      }
      tc_commit(&sh->drain);  // completes once every product issued above has
      const long long t0 = clock64();
      while (!mbar_try_wait(&sh->drain, 0) && clock64() - t0 < kRcWait) {
      }
    }
  } else if (warp < kRcSplitWarps) {
    // ----------------------------------------------------------- splitters
    long long g = 0, gh = 0;
    bool ok = true;
    for (long long i = 0; i < nmine && ok; ++i) {
      int ct, chunk, b, row0, nst;
      unit(i, ct, chunk, b, row0, nst);
      for (int s = 0; s < nst && ok; ++s, ++g) {
        const int q = (int)(g % kRcStages);
        // warp-uniform outcomes: the warp syncs below need every lane
        if (!__all_sync(0xffffffffu, rc_wait(&sh->full[q], (unsigned)((g / kRcStages) & 1), sh))) {
          ok = false;
          break;
        }
        const unsigned char *sx = base + q * kRcStageBytes, *sv = sx + kRcXBytes;
        for (int h = 0; h < 2; ++h, ++gh) {
          const int pb = (int)(gh & 1);
          if (gh >= 2 &&
              !__all_sync(0xffffffffu, rc_wait(&sh->planes_free[pb], (unsigned)(((gh >> 1) - 1) & 1), sh))) {
            ok = false;
            break;
          }
          unsigned char *px = planes + pb * kRcPlaneSet, *pv = px + 3 * kRcPX;
          // Stage line 2 j + h = rows 32 h .. 32 h + 31 of column j (128 bytes,
          // swizzled).  Task (j, c): its 16-byte chunk c = rows 4c .. 4c+3 of the
          // half, into plane row j, bytes 8c .. 8c+7 (8 lanes: one line; one row).
#pragma unroll
          for (int t = 0; t < 8 * kRcM / kSplitThreads; ++t) {
            const int task = tid + kSplitThreads * t, c = task & 7, j = task >> 3;
            const float4 v = *reinterpret_cast<const float4 *>(sx + swz128(2 * j + h, c));
            put_planes4(px, kRcPX, swz64(j, c >> 1) + 8 * (c & 1), v);
          }
          if (tid < 8 * kRcN) {  // V: rank qq, the same cut (one task per thread of the first 256)
            const int c = tid & 7, qq = tid >> 3;
            const float4 v = *reinterpret_cast<const float4 *>(sv + swz128(2 * qq + h, c));
            put_planes4(pv, kRcPV, swz64(qq, c >> 1) + 8 * (c & 1), v);
          }
          fence_proxy_async_smem();  // the planes are read by the tensor core (async proxy)
          __syncwarp();              // one arrival per warp, after every lane's writes
          if (lane == 0) mbar_arrive(&sh->planes_ready[pb]);
        }
        __syncwarp();  // every lane's reads of the stage are done
        if (ok && lane == 0) mbar_arrive(&sh->slot_free[q]);
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int w = warp - kEpi0, j = 32 * w + lane;  // accumulator row = column j of the tile
    long long grp = 0;
    for (long long i = 0; i < nmine; ++i) {
      int ct, chunk, b, row0, nst;
      unit(i, ct, chunk, b, row0, nst);
      float sum[kRcN];
#pragma unroll
      for (int q = 0; q < kRcN; ++q) sum[q] = 0.f;
      bool ok = true;
      const int ngrp = (2 * nst + kRcGroup - 1) / kRcGroup;
      for (int gi = 0; gi < ngrp; ++gi, ++grp) {
        const int ac = (int)(grp & 1);
        // warp-uniform outcome: tcgen05.ld is a warp-collective instruction
        if (!__all_sync(0xffffffffu, rc_wait(&sh->acc_full[ac], (unsigned)((grp >> 1) & 1), sh))) {
          ok = false;
          break;
        }
        tc_fence_after();
        const unsigned tl = tmem + ((unsigned)(32 * w) << 16) + (unsigned)(kRcAcc * ac);
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {  // ranks 16 hf .. 16 hf + 15 of the three blocks
          unsigned v[3][16];
#pragma unroll
          for (int blk = 0; blk < 3; ++blk) tc_ld16(tl + kRcN * blk + 16 * hf, v[blk]);
          tc_wait_ld(v);
#pragma unroll
          for (int q = 0; q < 16; ++q)
            sum[16 * hf + q] += (__uint_as_float(v[0][q]) + __uint_as_float(v[1][q])) + __uint_as_float(v[2][q]);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sh->acc_free[ac]);
      }
      if (!ok) break;
      const int jg = ct * kRcM + j;
      if (jg < a.C) {
        OutT *o = out + ((long long)b * a.nchunks + chunk) * a.r * a.C + (long long)jg * a.r;
#pragma unroll
        for (int q = 0; q < kRcN; ++q)
          if (q < a.r) o[q] = (OutT)sum[q];
      }
    }
  }
  __syncthreads();
  if (tid == 32 * kProd && sh->abort) {  // the producer thread
    report_error(a.st, HODLR_ERR_TIMEOUT, blockIdx.x);
    // loads issued but possibly still landing: wait (bounded) for them
    for (long long g = issued > kRcStages ? issued - kRcStages : 0; g < issued; ++g) {
      const long long t0 = clock64();
      while (!mbar_try_wait(&sh->full[g % kRcStages], (unsigned)((g / kRcStages) & 1)) &&
             clock64() - t0 < sh->budget) {
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMma) {
    tc_fence_after();
    tc_dealloc(tmem, kRcTmemCols);
  }
}

// The tcgen05 path of an FP32 row reduction, if its preconditions hold (else
// false): V is nrows*nbatch x r (r <= 32), X nrows*nbatch x C, both with
// 16-byte aligned bases and leading dimensions, rows and chunks multiples of 64.
template <typename OutT>
bool reduce_tc_try(const float *V, long long ldv, const float *X, long long ldx, long long nrows, int nbatch, int r,
                   int C, int chunk_rows, int nchunks, OutT *dst, const int *skip, DevStatus *st, cudaStream_t s,
                   cudaError_t &err) {
  const char *off = getenv("HODLR_NO_TCGEN05");
  if (off && off[0] == '1') return false;
  if (r < 1 || r > kRcN || C < 1 || nrows % kRcK || chunk_rows % kRcK || chunk_rows < kRcK) return false;
  const long long total = nrows * nbatch;
  if (total > 0x7fffffffLL) return false;  // tensor coordinates are 32-bit
  CUtensorMap mx, mv;
  if (!make_tensor_map_f32_rowblocks(&mx, X, total, C, ldx, kRcK / 32, kRcM)) return false;
  if (!make_tensor_map_f32_rowblocks(&mv, V, total, r, ldv, kRcK / 32, kRcN)) return false;
  auto k = reduce_tc_kernel<OutT>;
  static bool attr = false;
  if (!attr) {
    err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRcSmem);
    if (err != cudaSuccess) return true;
    attr = true;
  }
  RcArgs ra;
  ra.nrows = nrows;
  ra.nbatch = nbatch;
  ra.r = r;
  ra.C = C;
  ra.chunk_rows = chunk_rows;
  ra.nchunks = nchunks;
  ra.nct = ceil_div(C, kRcM);
  ra.nunits = (long long)ra.nct * nchunks * nbatch;
  ra.skip = skip;
  ra.st = st;
  const long long grid = persistent_ctas(ra.nunits);
  HODLR_LAUNCH(k, (unsigned)grid, kRcThreads, kRcSmem, s, mx, mv, ra, dst);
  err = cudaGetLastError();
  return true;
}

template bool reduce_tc_try<float>(const float *, long long, const float *, long long, long long, int, int, int, int,
                                   int, float *, const int *, DevStatus *, cudaStream_t, cudaError_t &);
template bool reduce_tc_try<double>(const float *, long long, const float *, long long, long long, int, int, int, int,
                                    int, double *, const int *, DevStatus *, cudaStream_t, cudaError_t &);

}  // namespace hodlr
