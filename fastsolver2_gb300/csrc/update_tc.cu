// K5 on the tcgen05 tensor cores: C_b -= U_b eta_b for the FP32 operands of
// the mixed path (rank <= 32), FP32-class accurate through an exact
// three-way bf16 split.
//
// Each FP32 operand x is cut into bf16 planes x = h + m + l (h = bf16(x),
// m = bf16(x - h), l = bf16(x - h - m): 24 significant bits; both
// subtractions are exact).  A product keeps the six terms down to relative
// size 2^-16 (hh, hm, mh, hl, mm, lh); the three dropped ones are below
// 2^-23 of |a b| together -- the accuracy class of an FP32 FMA (2^-24) --
// and the six accumulate in FP32 in tensor memory.  The tensor cores make
// the arithmetic small, so the kernel is a stream over 128-row x 64-column
// tiles of C: one persistent CTA per SM walks its tiles through a 3-stage
// ring of (U tile FP32 128 x 32, C tile FP32 128 x 64, eta tile FP32 32 x 64)
// with its steps split among warp roles (below) so that consecutive tiles
// overlap.  Waits are bounded; on timeout the CTA records HODLR_ERR_TIMEOUT,
// waits (bounded) for its copies and products and frees its tensor memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>

#include "kernels.cuh"
#include "tcgen05.cuh"
#include "tma.cuh"

namespace hodlr {

namespace {

constexpr int kBM = 128, kKS = 32;
constexpr int kABytes32 = kKS * kBM * 4;  // the FP32 U tile: 16 KB
constexpr int kPA = kBM * kKS * 2;        // one bf16 plane of the U tile: 8 KB

// Tiles of 128 rows x BN columns of C through a ring of STAGES stages.
template <int BN, int STAGES> struct UpdCfg {
  static constexpr int kCBytes = BN * kBM * 4;                         // the FP32 C tile
  static constexpr int kStageBytes = kABytes32 + kCBytes + BN * kKS * 4;  // + the FP32 eta tile
  static constexpr int kPB = BN * kKS * 2;                             // one bf16 plane of the eta tile
  static constexpr size_t kSmem = (size_t)STAGES * kStageBytes + 3 * kPA + 3 * kPB + 1024;
};

}  // namespace

// Warp roles joined by mbarriers instead of block barriers, so that tile
// i's epilogue, tile i+1's split and products and the loads of tile i+2 run
// at the same time.  SW warps cut the U and eta tiles into planes (written
// in the K-major 64-byte-swizzled layout the MMA descriptors read); one
// thread issues the 12 products (6 plane pairs x 2 K-steps, M 128, N 64,
// K 16) into one of two 64-column accumulators in tensor memory; four warps
// add alpha times the accumulator (tcgen05.ld) to the C tile in its stage;
// one thread issues the TMA loads and, once a tile's epilogue is done, its
// TMA store, refilling the stage after the store has read it.  Every wait
// is bounded and also ends when another role aborted.
namespace {

// warps 0 .. SW-1 split, SW .. SW+3 run the epilogue, SW+4 loads and
// stores, SW+5 issues the products
__host__ __device__ constexpr int ws_threads(int sw) { return 32 * (sw + 6); }
constexpr long long kWsWait = 2000000000LL;  // about one second of SM clocks
constexpr int kWsMaxStages = 8;

struct WsShared {
  uint64_t full[kWsMaxStages], tile_done[kWsMaxStages];
  uint64_t planes_ready, planes_free, acc_full[2], acc_free[2], drain;
  unsigned tmem;
  int abort;
};

__device__ __forceinline__ bool ws_wait(uint64_t *bar, unsigned parity, WsShared *sh) {
  return mbar_wait_or_abort(bar, parity, &sh->abort, kWsWait);
}

}  // namespace

template <int BN, int STAGES, int SW>
__global__ void __launch_bounds__(ws_threads(SW), 1)
update_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapC,
                 const __grid_constant__ CUtensorMap mapE, UpdateArgs a, int nrt, int nct, long long ntiles,
                 DevStatus *st) {
  if (a.skip && *a.skip) return;
  using WsCfg = UpdCfg<BN, STAGES>;
  static_assert(STAGES <= kWsMaxStages && (BN == 32 || BN == 64), "update_tc_kernel shape");
  constexpr int kBN = BN, kStages = STAGES, kStageBytes = WsCfg::kStageBytes, kPB = WsCfg::kPB;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char *pa = base + kStages * kStageBytes;  // 3 planes of the U tile
  unsigned char *pb = pa + 3 * kPA;                  // 3 planes of the eta tile
  __shared__ WsShared shm;
  WsShared *sh = &shm;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long nmine = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  auto tile_of = [&](long long i, int &rt, int &ct, int &b) {
    long long lin = blockIdx.x + i * gridDim.x;
    rt = (int)(lin % nrt);
    lin /= nrt;
    ct = (int)(lin % nct);
    b = (int)(lin / nct);
  };
  if (tid == 0) {
    prefetch_tensormap(&mapA);
    prefetch_tensormap(&mapC);
    prefetch_tensormap(&mapE);
    for (int q = 0; q < kStages; ++q) {
      mbar_init(&sh->full[q], 1);
      mbar_init(&sh->tile_done[q], 128);
    }
    mbar_init(&sh->planes_ready, 32 * SW);
    mbar_init(&sh->planes_free, 1);
    for (int q = 0; q < 2; ++q) {
      mbar_init(&sh->acc_full[q], 1);
      mbar_init(&sh->acc_free[q], 128);
    }
    mbar_init(&sh->drain, 1);
    sh->abort = 0;
    mbar_fence_init();
  }
  constexpr int kProd = SW + 4, kMmaWarp = SW + 5, kSplitThreads = 32 * SW;
  if (warp == kMmaWarp) {
    tc_alloc(&sh->tmem, 2 * kBN);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = sh->tmem;
  long long issued = 0;  // tiles whose loads were issued (producer)
  if (warp == kProd) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      auto store = [&](long long j) -> bool {
        const int s = (int)(j % kStages);
        if (!ws_wait(&sh->tile_done[s], (unsigned)((j / kStages) & 1), sh)) return false;
        int rt, ct, b;
        tile_of(j, rt, ct, b);
        tma_store_2d(&mapC, base + s * kStageBytes + kABytes32, (int)((long long)b * a.c_bstride + rt * kBM),
                     ct * kBN);
        tma_store_commit();
        return true;
      };
      for (long long j = 0; j < nmine; ++j) {
        const int s = (int)(j % kStages);
        if (j >= kStages) {  // stage s last held tile j - kStages: store it, let the store read it
          if (!store(j - kStages)) break;
          tma_store_wait_read_all();
        }
        int rt, ct, b;
        tile_of(j, rt, ct, b);
        unsigned char *sa = base + s * kStageBytes;
        mbar_arrive_expect_tx(&sh->full[s], kStageBytes);
        tma_load_2d(sa, &mapA, &sh->full[s], (int)((long long)b * a.a_bstride + rt * kBM), 0);
        tma_load_2d(sa + kABytes32, &mapC, &sh->full[s], (int)((long long)b * a.c_bstride + rt * kBM), ct * kBN);
        tma_load_2d(sa + kABytes32 + WsCfg::kCBytes, &mapE, &sh->full[s], (int)(((b & 1) ^ a.b_flip) * a.b_s2),
                    (int)((long long)(b >> 1) * a.N + ct * kBN));
        issued = j + 1;
      }
      for (long long j = issued > kStages ? issued - kStages : 0; j < issued && !sh->abort; ++j)
        if (!store(j)) break;
      tma_store_wait_read_all();
    }
  } else if (warp == kMmaWarp) {
    // ---------------------------------------------------------------- MMA
    if (lane == 0) {
      const unsigned idesc = tc_idesc_bf16(kBM, kBN);
      const int ps[6] = {0, 0, 1, 0, 1, 2}, pt[6] = {0, 1, 0, 2, 1, 0};
      for (long long i = 0; i < nmine; ++i) {
        const int ac = (int)(i & 1);
        if (!ws_wait(&sh->planes_ready, (unsigned)(i & 1), sh)) break;
        if (i >= 2 && !ws_wait(&sh->acc_free[ac], (unsigned)(((i >> 1) - 1) & 1), sh)) break;
        tc_fence_after();
        const unsigned d = tmem + (unsigned)(kBN * ac);
#pragma unroll
        for (int kk = 0; kk < 2; ++kk)
#pragma unroll
          for (int u = 0; u < 6; ++u)
            tc_mma(d, desc_sw64(smem_u32(pa + ps[u] * kPA)) + 2 * kk, desc_sw64(smem_u32(pb + pt[u] * kPB)) + 2 * kk,
                   idesc, (kk > 0 || u > 0) ? 1u : 0u);
        tc_commit(&sh->acc_full[ac]);
        tc_commit(&sh->planes_free);
      }
      tc_commit(&sh->drain);  // completes once every product issued above has
      const long long t0 = clock64();
      while (!mbar_try_wait(&sh->drain, 0) && clock64() - t0 < kWsWait) {
      }
    }
  } else if (warp < SW) {
    // ----------------------------------------------------------- splitters
    for (long long i = 0; i < nmine; ++i) {
      const int s = (int)(i % kStages);
      if (!ws_wait(&sh->full[s], (unsigned)((i / kStages) & 1), sh)) break;
      if (i >= 1 && !ws_wait(&sh->planes_free, (unsigned)((i - 1) & 1), sh)) break;
      int rt, ct, b;
      tile_of(i, rt, ct, b);
      const float *sA = reinterpret_cast<const float *>(base + s * kStageBytes);  // [kKS][kBM]
      const float *sE = reinterpret_cast<const float *>(base + s * kStageBytes + kABytes32 + WsCfg::kCBytes);
      constexpr int kEtaTasks = 4 * kBN;  // column j of C, 8 K values per task (fewer tasks than threads at BN 32)
#pragma unroll
      for (int t = 0; t < (kEtaTasks + kSplitThreads - 1) / kSplitThreads; ++t) {  // eta planes
        const int task = tid + kSplitThreads * t, j = task >> 2, c = task & 3, jg = ct * kBN + j;
        if (task >= kEtaTasks) continue;
        const float4 e0 = *reinterpret_cast<const float4 *>(sE + j * kKS + 8 * c);
        const float4 e1 = *reinterpret_cast<const float4 *>(sE + j * kKS + 8 * c + 4);
        float x[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
#pragma unroll
        for (int e = 0; e < 8; ++e)
          if (8 * c + e >= a.K || jg >= a.N) x[e] = 0.f;
        put_planes(pb, kPB, swz64(j, c), x);
      }
#pragma unroll
      for (int t = 0; t < 4 * kBM / kSplitThreads; ++t) {  // U planes: consecutive lanes take consecutive rows
        const int task = tid + kSplitThreads * t, r = task & (kBM - 1), c = task >> 7;
        float x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = sA[(8 * c + e) * kBM + r];
        put_planes(pa, kPA, swz64(r, c), x);
      }
      fence_proxy_async_smem();  // the planes are read by the tensor core (async proxy)
      mbar_arrive(&sh->planes_ready);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp - SW, r = 32 * q + lane;
    const float alpha = (float)a.alpha;
    for (long long i = 0; i < nmine; ++i) {
      const int s = (int)(i % kStages), ac = (int)(i & 1);
      // warp-uniform outcomes: tcgen05.ld below is a warp-collective instruction
      if (!__all_sync(0xffffffffu, ws_wait(&sh->acc_full[ac], (unsigned)((i >> 1) & 1), sh))) break;
      if (!__all_sync(0xffffffffu, ws_wait(&sh->full[s], (unsigned)((i / kStages) & 1), sh))) break;  // C landed
      tc_fence_after();
      unsigned v[kBN / 32][32];
      const unsigned tl = tmem + ((unsigned)(32 * q) << 16) + (unsigned)(kBN * ac);
#pragma unroll
      for (int h = 0; h < kBN / 32; ++h) tc_ld32(tl + 32 * h, v[h]);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      tc_fence_before();
      mbar_arrive(&sh->acc_free[ac]);
      float *sC = reinterpret_cast<float *>(base + s * kStageBytes + kABytes32);  // [kBN][kBM]
#pragma unroll
      for (int h = 0; h < kBN / 32; ++h)
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          float *cp = sC + (32 * h + c) * kBM + r;
          *cp = fmaf(alpha, __uint_as_float(v[h][c]), *cp);
        }
      fence_proxy_async_smem();  // the C tile is read by the TMA store (async proxy)
      mbar_arrive(&sh->tile_done[s]);
    }
  }
  __syncthreads();
  if (tid == 32 * kProd && sh->abort) {  // the producer thread
    report_error(st, HODLR_ERR_TIMEOUT, blockIdx.x);
    // loads issued but possibly still landing: wait (bounded) for them
    for (long long j = issued > kStages ? issued - kStages : 0; j < issued; ++j) {
      const long long t0 = clock64();
      while (!mbar_try_wait(&sh->full[j % kStages], (unsigned)((j / kStages) & 1)) && clock64() - t0 < kWsWait) {
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    tc_dealloc(tmem, 2 * kBN);
  }
}

template <int BN, int STAGES, int SW>
static cudaError_t update_tc_launch(const UpdateArgs &a, DevStatus *st, cudaStream_t s, bool &done) {
  using WsCfg = UpdCfg<BN, STAGES>;
  constexpr int kWsBN = BN;
  done = false;
  const long long rows = (long long)a.M * a.nbatch;
  CUtensorMap ma, mc, me;
  if (!make_tensor_map_f32(&ma, static_cast<const float *>(a.A), rows, a.K, a.lda, kBM, kKS, false))
    return cudaSuccess;
  if (!make_tensor_map_f32(&mc, static_cast<const float *>(a.C), rows, a.N, a.ldc, kBM, kWsBN, false))
    return cudaSuccess;
  if (!make_tensor_map_f32(&me, a.B32, a.ldb, (long long)(a.nbatch / 2) * a.N, a.ldb, kKS, kWsBN, false))
    return cudaSuccess;
  done = true;
  const int nrt = a.M / kBM, nct = (a.N + kWsBN - 1) / kWsBN;
  auto k = update_tc_kernel<BN, STAGES, SW>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WsCfg::kSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long long ntiles = (long long)nrt * nct * a.nbatch;
  const long long grid = persistent_ctas(ntiles);
  HODLR_LAUNCH(k, (unsigned)grid, ws_threads(SW), WsCfg::kSmem, s, ma, mc, me, a, nrt, nct, ntiles, st);
  return cudaGetLastError();
}

// The tcgen05 path for an FP32 update, if its preconditions hold (else false).
bool update_tc_try(const UpdateArgs &a, DevStatus *st, cudaStream_t s, cudaError_t &err) {
  const char *off = getenv("HODLR_NO_TCGEN05");
  if (off && off[0] == '1') return false;
  if (a.a_trans || !a.B32 || a.b_trans || a.K < 1 || a.K > kKS || a.a_bstride != a.M || a.c_bstride != a.M ||
      a.M % kBM || a.nbatch % 2 || a.b_s1 != (long long)a.ldb * a.N || a.b_s2 % 4 || a.ldb < 2 * a.b_s2)
    return false;
  bool done = false;
  switch (current_tuning().upd_tc_shape) {
    case 1: err = update_tc_launch<64, 2, 8>(a, st, s, done); break;
    case 2: err = update_tc_launch<32, 5, 8>(a, st, s, done); break;
    default: err = update_tc_launch<64, 3, 8>(a, st, s, done); break;
  }
  return done || err != cudaSuccess;
}

}  // namespace hodlr
