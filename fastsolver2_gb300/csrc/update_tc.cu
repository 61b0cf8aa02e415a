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
// ring, TMA bringing the U tile (FP32, 128 x 32) and the C tile (FP32,
// 128 x 64) of tiles i+1 and i+2 while tile i is processed -- its eta block
// and U tile split into planes (written in the K-major 64-byte-swizzled
// layout the MMA descriptors read), one thread issuing the 12 MMAs (6
// products x 2 K-steps, M 128, N 64, K 16) into a 64-column tensor-memory
// accumulator, eight warps adding alpha times it (tcgen05.ld) to the C tile
// in its stage, and one TMA store writing it back; a stage is refilled once
// its store has read it.  Waits are bounded; on timeout the CTA records
// HODLR_ERR_TIMEOUT, waits (bounded) for its copies and products and frees
// its tensor memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>

#include "kernels.cuh"
#include "tcgen05.cuh"
#include "tma.cuh"

namespace hodlr {

namespace {

constexpr int kBM = 128, kBN = 64, kKS = 32;
constexpr int kStages = 3;                     // ring of (U tile, C tile) stages
constexpr int kABytes32 = kKS * kBM * 4;       // the FP32 U tile: 16 KB
constexpr int kCBytes32 = kBN * kBM * 4;       // the FP32 C tile: 32 KB
constexpr int kStageBytes = kABytes32 + kCBytes32 + kBN * kKS * 4;  // + the FP32 eta tile: 56 KB
constexpr int kPA = kBM * kKS * 2;  // one bf16 plane of the U tile: 8 KB
constexpr int kPB = kBN * kKS * 2;  // one bf16 plane of the eta tile: 4 KB
constexpr size_t kSmem = (size_t)kStages * kStageBytes + 3 * kPA + 3 * kPB + 1024;

}  // namespace

__global__ void __launch_bounds__(256, 1)
update_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapC,
                 const __grid_constant__ CUtensorMap mapE, UpdateArgs a, int nrt, int nct, long long ntiles,
                 DevStatus *st) {
  if (a.skip && *a.skip) return;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char *pa = base + kStages * kStageBytes;  // 3 planes of the U tile
  unsigned char *pb = pa + 3 * kPA;                  // 3 planes of the eta tile
  __shared__ __align__(8) uint64_t full[kStages], mma_bar;
  __shared__ unsigned s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // this CTA's tiles: blockIdx.x, blockIdx.x + gridDim.x, ...
  const long long nmine = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  auto tile_of = [&](long long i, int &rt, int &ct, int &b) {
    long long lin = blockIdx.x + i * gridDim.x;
    rt = (int)(lin % nrt);
    lin /= nrt;
    ct = (int)(lin % nct);
    b = (int)(lin / nct);
  };
  auto issue = [&](long long i) {  // thread 0: loads of tile i into stage i % kStages
    int rt, ct, b;
    tile_of(i, rt, ct, b);
    const int sidx = (int)(i % kStages);
    unsigned char *sa = base + sidx * kStageBytes;
    mbar_arrive_expect_tx(&full[sidx], kStageBytes);
    tma_load_2d(sa, &mapA, &full[sidx], (int)((long long)b * a.a_bstride + rt * kBM), 0);
    tma_load_2d(sa + kABytes32, &mapC, &full[sidx], (int)((long long)b * a.c_bstride + rt * kBM), ct * kBN);
    // eta of child b: rows ((b & 1) ^ flip) r .. of node b >> 1's block, columns ct * kBN ..
    tma_load_2d(sa + kABytes32 + kCBytes32, &mapE, &full[sidx], (int)(((b & 1) ^ a.b_flip) * a.b_s2),
                (int)((long long)(b >> 1) * a.N + ct * kBN));
  };
  if (tid == 0) {
    prefetch_tensormap(&mapA);
    prefetch_tensormap(&mapC);
    prefetch_tensormap(&mapE);
    for (int q = 0; q < kStages; ++q) mbar_init(&full[q], 1);
    mbar_init(&mma_bar, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tc_alloc(&s_tmem, 64);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = s_tmem;
  if (tid == 0)
    for (long long i = 0; i < nmine && i < kStages - 1; ++i) issue(i);
  const unsigned idesc = tc_idesc_bf16(kBM, kBN);
  const float alpha = (float)a.alpha;
  long long done = 0;  // tiles finished
  bool ok = true;
  for (long long i = 0; i < nmine; ++i) {
    int rt, ct, b;
    tile_of(i, rt, ct, b);
    const int sidx = (int)(i % kStages);
    float *sA = reinterpret_cast<float *>(base + sidx * kStageBytes);  // [kKS][kBM]
    float *sC = sA + kKS * kBM;                                         // [kBN][kBM]
    if (tid == 0 && i + kStages - 1 < nmine) {
      // the stage of tile i + 2 last held tile i - 1: its store must have read it
      tma_store_wait_read_all();
      issue(i + kStages - 1);
    }
    bool got = mbar_wait_bounded(&full[sidx], (unsigned)((i / kStages) & 1));
    if (got) {
      // eta planes of this tile: row j (a column of C), 8 K values per thread;
      // rows beyond the rank and columns beyond the block are zero
      const float *sE = reinterpret_cast<const float *>(base + sidx * kStageBytes + kABytes32 + kCBytes32);
      // eta planes: 8 consecutive K values of column j (two 16-byte loads;
      // a quarter warp reads 128 contiguous bytes)
      const int j = tid >> 2, c = tid & 3, jg = ct * kBN + j;
      const float4 e0 = *reinterpret_cast<const float4 *>(sE + j * kKS + 8 * c);
      const float4 e1 = *reinterpret_cast<const float4 *>(sE + j * kKS + 8 * c + 4);
      float x[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
#pragma unroll
      for (int e = 0; e < 8; ++e)
        if (8 * c + e >= a.K || jg >= a.N) x[e] = 0.f;
      put_planes(pb, kPB, swz64(j, c), x);
#pragma unroll
      for (int t = 0; t < 2; ++t) {  // U planes: row r of the tile, 8 K values per task
        // consecutive lanes take consecutive rows: conflict-free column reads
        const int task = tid + 256 * t, r = task & (kBM - 1), c = task >> 7;
        float x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = sA[(8 * c + e) * kBM + r];
        put_planes(pa, kPA, swz64(r, c), x);
      }
    }
    fence_proxy_async_smem();  // the planes are read by the tensor core (async proxy)
    tc_fence_before();
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    tc_fence_after();
    if (tid == 0) {
      // the six products of the planes with terms down to 2^-16, over two K-steps of 16
      const int ps[6] = {0, 0, 1, 0, 1, 2}, pt[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
      for (int kk = 0; kk < 2; ++kk)
#pragma unroll
        for (int u = 0; u < 6; ++u)
          tc_mma(tmem, desc_sw64(smem_u32(pa + ps[u] * kPA)) + 2 * kk,
                 desc_sw64(smem_u32(pb + pt[u] * kPB)) + 2 * kk, idesc, (kk > 0 || u > 0) ? 1u : 0u);
      tc_commit(&mma_bar);
    }
    const bool fin = mbar_wait_bounded(&mma_bar, (unsigned)(i & 1));
    if (__syncthreads_or(!fin)) {
      ok = false;
      break;
    }
    tc_fence_after();
    {
      // warp w: rows 32 (w % 4) + lane of the tile, columns 32 (w / 4) ..
      const int q = warp & 3, h = warp >> 2, r = 32 * q + lane;
      unsigned v[32];
      tc_ld32(tmem + ((unsigned)(32 * q) << 16) + (unsigned)(32 * h), v);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        float *cp = sC + (32 * h + c) * kBM + r;
        float d;
        asm volatile("mov.b32 %0, %1;" : "=f"(d) : "r"(v[c]));
        *cp = fmaf(alpha, d, *cp);
      }
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();  // also: every thread is done with the planes and the tensor memory of tile i
    if (tid == 0) {
      tma_store_2d(&mapC, sC, (int)((long long)b * a.c_bstride + rt * kBM), ct * kBN);
      tma_store_commit();
    }
    ++done;
  }
  if (tid == 0) {
    if (!ok) {
      report_error(st, HODLR_ERR_TIMEOUT, blockIdx.x);
      // copies issued for tiles not finished, and the last products: wait for them (bounded)
      for (long long i = done; i < nmine && i < done + kStages; ++i)
        (void)mbar_wait_bounded(&full[i % kStages], (unsigned)((i / kStages) & 1));
      (void)mbar_wait_bounded(&mma_bar, (unsigned)(done & 1));
    }
    tma_store_wait_read_all();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_dealloc(tmem, 64);
  }
}

// The tcgen05 path for an FP32 update, if its preconditions hold (else false).
bool update_tc_try(const UpdateArgs &a, DevStatus *st, cudaStream_t s, cudaError_t &err) {
  const char *off = getenv("HODLR_NO_TCGEN05");
  if (off && off[0] == '1') return false;
  if (a.a_trans || !a.B32 || a.b_trans || a.K < 1 || a.K > kKS || a.a_bstride != a.M || a.c_bstride != a.M ||
      a.M % kBM || a.nbatch % 2 || a.b_s1 != (long long)a.ldb * a.N || a.b_s2 % 4 || a.ldb < 2 * a.b_s2)
    return false;
  const long long rows = (long long)a.M * a.nbatch;
  CUtensorMap ma, mc;
  if (!make_tensor_map_f32(&ma, static_cast<const float *>(a.A), rows, a.K, a.lda, kBM, kKS, false)) return false;
  if (!make_tensor_map_f32(&mc, static_cast<const float *>(a.C), rows, a.N, a.ldc, kBM, kBN, false)) return false;
  // eta of every node as one matrix: ldb rows (both children's blocks), N columns per node
  CUtensorMap me;
  if (!make_tensor_map_f32(&me, a.B32, a.ldb, (long long)(a.nbatch / 2) * a.N, a.ldb, kKS, kBN, false)) return false;
  const int nrt = a.M / kBM, nct = (a.N + kBN - 1) / kBN;
  static bool attr = false;
  if (!attr) {
    err = cudaFuncSetAttribute(update_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    if (err != cudaSuccess) return true;
    attr = true;
  }
  const long long ntiles = (long long)nrt * nct * a.nbatch;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long grid = std::min<long long>(ntiles, sms > 0 ? sms : 148);
  HODLR_LAUNCH(update_tc_kernel, (unsigned)grid, 256, kSmem, s, ma, mc, me, a, nrt, nct, ntiles, st);
  err = cudaGetLastError();
  return true;
}

}  // namespace hodlr
