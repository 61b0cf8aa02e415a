// K3 / K5: the batched tall-skinny GEMMs of the sweep.
//
//   K3 reduce_tn  Out_b = A_b^T X_b   (r x C per child; A_b, X_b = the child's
//                 rows of V^(l) or Utilde^(l) and of the right-hand sides) --
//                 the V^T [u|d] products of hsolve (src/tasks/leaf_solve.cc:
//                 132-135) and GemmRedTask (src/tasks/gemm_reduce.cc:33-83).
//   K5 update_nn  C_b += alpha A_b diag(s) op(B_b) -- d -= u eta of hsolve
//                 (leaf_solve.cc:143-153) and GemmBroTask
//                 (src/tasks/gemm_broadcast.cc:33-83); the tree's
//                 child/sibling/node indexing is folded into the batch
//                 addressing of B.
//
// K3 splits the long row dimension three ways: across CTAs (row chunks,
// summed by a deterministic second pass -- no atomics, so results are bitwise
// reproducible run to run), across the four 64-thread groups of a CTA (summed
// in shared memory in a fixed order), and along each thread's rows.  Each
// thread keeps an (RT/8) x 8 register tile; shared-memory rows are padded by
// one element so the column-wise staging stores are bank-conflict free.
#include <algorithm>
#include <type_traits>

#include "kernels.cuh"
#include "tma.cuh"

namespace hodlr {

// ------------------------------------------------------------ tensor maps
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      (void)cudaGetLastError();
      return (EncodeTiledFn) nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

bool make_tensor_map_f32(CUtensorMap *map, const float *base, long long rows, long long cols, long long ld,
                         int box_rows, int box_cols, bool swizzle128) {
  EncodeTiledFn f = encode_fn();
  if (!f || !base || rows < 1 || cols < 1) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld * 4) % 16 || ld < rows) return false;
  cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
  cuuint32_t box[2] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols};
  cuuint32_t es[2] = {1, 1};
  return f(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_tensor_map_f64(CUtensorMap *map, const double *base, long long rows, long long cols, long long ld,
                         int box_rows, int box_cols) {
  EncodeTiledFn f = encode_fn();
  if (!f || !base || rows < 1 || cols < 1) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld * 8) % 16 || ld < rows) return false;
  cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 8};
  cuuint32_t box[2] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols};
  cuuint32_t es[2] = {1, 1};
  return f(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double *>(base), dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_tensor_map_f32_rowblocks(CUtensorMap *map, const float *base, long long rows, long long cols, long long ld,
                                   int row_blocks, int box_cols) {
  EncodeTiledFn f = encode_fn();
  if (!f || !base || rows < 32 || rows % 32 || cols < 1) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld * 4) % 16 || ld < rows) return false;
  cuuint64_t dims[3] = {32, (cuuint64_t)(rows / 32), (cuuint64_t)cols};
  cuuint64_t strides[2] = {128, (cuuint64_t)ld * 4};
  cuuint32_t box[3] = {32, (cuuint32_t)row_blocks, (cuuint32_t)box_cols};
  cuuint32_t es[3] = {1, 1, 1};
  return f(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_tensor_map_bf16(CUtensorMap *map, const void *base, long long inner, long long outer, long long ld,
                          int box_inner, int box_outer, int swizzle_bytes) {
  EncodeTiledFn f = encode_fn();
  if (!f || !base || inner < 1 || outer < 1) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld * 2) % 16 || ld < inner) return false;
  if (box_inner * 2 > swizzle_bytes && swizzle_bytes > 0) return false;
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_outer};
  cuuint32_t es[2] = {1, 1};
  const CUtensorMapSwizzle sw = swizzle_bytes == 128  ? CU_TENSOR_MAP_SWIZZLE_128B
                                : swizzle_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                : swizzle_bytes == 32 ? CU_TENSOR_MAP_SWIZZLE_32B
                                                      : CU_TENSOR_MAP_SWIZZLE_NONE;
  return f(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// ------------------------------------------------------------------ K3
// output columns per CTA: 64, or 8 for narrow right-hand sides (C <= 8)
static inline int red_bn(int C) { return C <= 8 ? 8 : 64; }
static constexpr int kRedBK = 32;   // rows staged per step
static thread_local const Tuning *g_tuning = nullptr;
static const Tuning kDefaultTuning{};
const Tuning &current_tuning() { return g_tuning ? *g_tuning : kDefaultTuning; }

long long persistent_ctas(long long units) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::max<long long>(1, std::min<long long>(units, sms > 0 ? sms : kNumSMs));
}
TuningScope::TuningScope(const Tuning *t) : prev(g_tuning) { g_tuning = t; }
TuningScope::~TuningScope() { g_tuning = prev; }

template <typename T, int RT, int BN, typename OutT>
__global__ void __launch_bounds__(256)
reduce_tn_kernel(const T *__restrict__ A, long long lda, const T *__restrict__ X, long long ldx,
                 long long nrows, int r, int C, int chunk_rows, int nchunks, int nct, OutT *out,
                 const int *skip) {
  if (skip && *skip) return;
  constexpr int RPT = RT / 8;           // ranks per thread (rows of the output)
  constexpr int CPT = BN / 8;           // columns per thread
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sA = reinterpret_cast<T *>(smem_raw);          // [kRedBK][RT]
  T *sX = sA + kRedBK * (RT + 1);                   // [kRedBK][BN + 1]
  T *sRed = sX + kRedBK * (BN + 1);                 // [4][RT][BN + 1]
  long long lin = blockIdx.x;
  const int ct = (int)(lin % nct);
  lin /= nct;
  const int chunk = (int)(lin % nchunks);
  const int b = (int)(lin / nchunks);
  const int c0 = ct * BN;
  const long long row_begin = (long long)b * nrows + (long long)chunk * chunk_rows;
  const int rows = (int)min((long long)chunk_rows, nrows - (long long)chunk * chunk_rows);
  const int tid = threadIdx.x, g = tid >> 6, t = tid & 63, tr = t & 7, tc = t >> 3;
  T acc[RPT][CPT];
#pragma unroll
  for (int a = 0; a < RPT; ++a)
#pragma unroll
    for (int c = 0; c < CPT; ++c) acc[a][c] = T(0);
  const T *Ab = A + row_begin;
  const T *Xb = X + row_begin + (long long)c0 * ldx;
  for (int i0 = 0; i0 < rows; i0 += kRedBK) {
    const int ib = min(kRedBK, rows - i0);
    for (int e = tid; e < kRedBK * RT; e += 256) {
      const int i = e % kRedBK, q = e / kRedBK;
      sA[i * (RT + 1) + q] = (i < ib && q < r) ? Ab[i0 + i + (long long)q * lda] : T(0);
    }
    for (int e = tid; e < kRedBK * BN; e += 256) {
      const int i = e % kRedBK, j = e / kRedBK;
      sX[i * (BN + 1) + j] = (i < ib && c0 + j < C) ? Xb[i0 + i + (long long)j * ldx] : T(0);
    }
    __syncthreads();
#pragma unroll 2
    for (int ii = 0; ii < kRedBK / 4; ++ii) {
      const int i = ii * 4 + g;
      T av[RPT], xv[CPT];
#pragma unroll
      for (int a = 0; a < RPT; ++a) av[a] = sA[i * (RT + 1) + tr * RPT + a];
#pragma unroll
      for (int c = 0; c < CPT; ++c) xv[c] = sX[i * (BN + 1) + tc * CPT + c];
#pragma unroll
      for (int a = 0; a < RPT; ++a)
#pragma unroll
        for (int c = 0; c < CPT; ++c) acc[a][c] += av[a] * xv[c];
    }
    __syncthreads();
  }
  // fixed-order sum of the four row groups
#pragma unroll
  for (int a = 0; a < RPT; ++a)
#pragma unroll
    for (int c = 0; c < CPT; ++c) sRed[(g * RT + tr * RPT + a) * (BN + 1) + tc * CPT + c] = acc[a][c];
  __syncthreads();
  OutT *o = out + ((long long)b * nchunks + chunk) * r * C;
  for (int e = tid; e < RT * BN; e += 256) {
    const int q = e % RT, j = e / RT;
    if (q >= r || c0 + j >= C) continue;
    double s = 0.0;
#pragma unroll
    for (int gg = 0; gg < 4; ++gg) s += (double)sRed[(gg * RT + q) * (BN + 1) + j];
    o[q + (long long)(c0 + j) * r] = (OutT)s;
  }
}

// K3, FP32 operands, TMA pipeline.  Each CTA owns one (column tile, row
// chunk) of one child block and streams its rows in stages of 32: one thread
// issues two 2-D TMA loads per stage (A: 32 rows x RT ranks, X: 32 rows x 64
// columns, both landing K-major with the 128-byte swizzle) into a 4-deep ring
// of shared-memory slots, completing on per-slot mbarriers.  The four 64-thread
// groups each take 8 of a stage's 32 rows; a thread reads float4 runs of 4
// rows for its RT/8 ranks (strided by 8: conflict-free under the swizzle) and
// 8 columns (broadcast within a quarter warp) and accumulates RT/8 x 8
// outputs.  The groups are summed in a fixed order at the end.
// Preconditions (checked on the host): block rows and chunk rows multiples
// of 32, 16-byte aligned bases and leading dimensions.
static constexpr int kTmaStages = 4;

// Test hook of the bounded waits (struct WaitFault, kernels.cuh), this
// kernel's copy.
__device__ WaitFault g_wait_fault = {-1, -1, 0};

// Stage s of a reduce CTA: rows [row0 + 32 s, +32) of A (all ranks) and of
// the X column tile at c0, into ring slot s % kTmaStages.
template <int A_BYTES, int STAGE>
__device__ __forceinline__ void reduce_tma_issue(unsigned char *base, uint64_t *bars, const CUtensorMap *mapA,
                                                 const CUtensorMap *mapX, int s, int row0, int c0) {
  const int slot = s % kTmaStages;
  unsigned char *sa = base + slot * STAGE;
  mbar_arrive_expect_tx(&bars[slot], STAGE);
  tma_load_2d(sa, mapA, &bars[slot], row0 + s * 32, 0);
  tma_load_2d(sa + A_BYTES, mapX, &bars[slot], row0 + s * 32, c0);
}

template <int RT, typename OutT>
__global__ void __launch_bounds__(256, RT <= 16 ? 3 : (RT <= 32 ? 2 : 1))
reduce_tma_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapX,
                  long long nrows, int r, int C, int chunk_rows, int nchunks, int nct, OutT *out,
                  const int *skip, DevStatus *st) {
  if (skip && *skip) return;
  constexpr int BN = 64, BK = 32, RPT = RT / 8, CPT = BN / 8;
  constexpr int A_BYTES = BK * RT * 4, X_BYTES = BK * BN * 4, STAGE = A_BYTES + X_BYTES;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) uint64_t bars[kTmaStages];
  long long lin = blockIdx.x;
  const int ct = (int)(lin % nct);
  lin /= nct;
  const int chunk = (int)(lin % nchunks);
  const int b = (int)(lin / nchunks);
  const int c0 = ct * BN;
  const long long row0 = (long long)b * nrows + (long long)chunk * chunk_rows;
  const int rows = (int)min((long long)chunk_rows, nrows - (long long)chunk * chunk_rows);
  const int nst = rows / BK;
  const int tid = threadIdx.x, g = tid >> 6, t = tid & 63, tr = t & 7, tc = t >> 3;
  if (tid == 0) {
    prefetch_tensormap(&mapA);
    prefetch_tensormap(&mapX);
    for (int q = 0; q < kTmaStages; ++q) mbar_init(&bars[q], 1);
    mbar_fence_init();
  }
  __syncthreads();
  const int row0i = (int)row0;  // tensor coordinates are 32-bit
  const WaitFault wf = g_wait_fault;
  const int skip_stage = wf.cta == (int)blockIdx.x ? wf.stage : -1;
  const long long budget = skip_stage >= 0 && wf.budget > 0 ? wf.budget : 1000000000LL;
  if (tid == 0)
    for (int s = 0; s < min(kTmaStages, nst); ++s)
      if (s != skip_stage) reduce_tma_issue<A_BYTES, STAGE>(base, bars, &mapA, &mapX, s, row0i, c0);
  // packed pair accumulators: .x sums the even rows of the chunk, .y the odd
  // ones (a float4 run holds both), so one packed FMA does two products
  float2 acc[RPT][CPT];
#pragma unroll
  for (int a = 0; a < RPT; ++a)
#pragma unroll
    for (int c = 0; c < CPT; ++c) acc[a][c] = make_float2(0.f, 0.f);
  for (int s = 0; s < nst; ++s) {
    const int slot = s % kTmaStages;
    const bool ok = mbar_wait_bounded(&bars[slot], (unsigned)((s / kTmaStages) & 1), budget);
    if (__syncthreads_or(!ok)) {  // every thread leaves together
      if (tid == 0) {
        report_error(st, HODLR_ERR_TIMEOUT, blockIdx.x);
        // copies still in flight: stages s .. max(kTmaStages, s + kTmaStages - 1) - 1
        // were issued (stage s + kTmaStages - 1 is issued only after stage s's wait)
        const int issued_end = min(nst, max(kTmaStages, s + kTmaStages - 1));
        for (int q = s; q < issued_end; ++q)
          (void)mbar_wait_bounded(&bars[q % kTmaStages], (unsigned)((q / kTmaStages) & 1), budget);
      }
      return;
    }
    // every thread has finished stage s-1: its slot can be refilled
    if (tid == 0 && s >= 1 && s - 1 + kTmaStages < nst && s - 1 + kTmaStages != skip_stage)
      reduce_tma_issue<A_BYTES, STAGE>(base, bars, &mapA, &mapX, s - 1 + kTmaStages, row0i, c0);
    const unsigned char *sa = base + slot * STAGE, *sx = sa + A_BYTES;
#pragma unroll
    for (int kc = 2 * g; kc < 2 * g + 2; ++kc) {
      float4 av[RPT];
#pragma unroll
      for (int a = 0; a < RPT; ++a) av[a] = *reinterpret_cast<const float4 *>(sa + swz128(tr + 8 * a, kc));
#pragma unroll
      for (int c = 0; c < CPT; ++c) {  // one column at a time keeps the live set small
        const float4 xv = *reinterpret_cast<const float4 *>(sx + swz128(tc + 8 * c, kc));
#pragma unroll
        for (int a = 0; a < RPT; ++a) {
          float2 v = acc[a][c];
          v = __ffma2_rn(make_float2(av[a].x, av[a].y), make_float2(xv.x, xv.y), v);
          v = __ffma2_rn(make_float2(av[a].z, av[a].w), make_float2(xv.z, xv.w), v);
          acc[a][c] = v;
        }
      }
    }
  }
  __syncthreads();  // all stages consumed: the ring becomes the group-sum buffer
  float *sRed = reinterpret_cast<float *>(base);  // [4][RT][BN + 1]
#pragma unroll
  for (int a = 0; a < RPT; ++a)
#pragma unroll
    for (int c = 0; c < CPT; ++c) sRed[(g * RT + tr + 8 * a) * (BN + 1) + tc + 8 * c] = acc[a][c].x + acc[a][c].y;
  __syncthreads();
  OutT *o = out + ((long long)b * nchunks + chunk) * r * C;
  for (int e = tid; e < RT * BN; e += 256) {
    const int q = e % RT, j = e / RT;
    if (q >= r || c0 + j >= C) continue;
    float sum = 0.f;  // fixed-order FP32 sum of the groups
#pragma unroll
    for (int gg = 0; gg < 4; ++gg) sum += sRed[(gg * RT + q) * (BN + 1) + j];
    o[q + (long long)(c0 + j) * r] = (OutT)sum;
  }
}

template <int RT>
static size_t reduce_tma_smem() {
  const size_t ring = (size_t)kTmaStages * 32 * (RT + 64) * 4, red = 4ull * RT * 65 * 4;
  return std::max(ring, red) + 1024;
}

template <int RT, typename OutT>
static cudaError_t reduce_tma_rt(const CUtensorMap &ma, const CUtensorMap &mx, long long nrows, int nbatch, int r,
                                 int C, int chunk_rows, int nchunks, int nct, OutT *dst, const int *skip,
                                 DevStatus *st, cudaStream_t s) {
  const size_t bytes = reduce_tma_smem<RT>();
  auto k = reduce_tma_kernel<RT, OutT>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long long nblk = (long long)nct * nchunks * nbatch;
  HODLR_LAUNCH(k, (unsigned)nblk, 256, bytes, s, ma, mx, nrows, r, C, chunk_rows, nchunks, nct, dst, skip, st);
  return cudaGetLastError();
}

// The TMA path for FP32 operands, if its preconditions hold (else false).
template <typename OutT>
static bool reduce_tma_try(const float *A, long long lda, const float *X, long long ldx, long long nrows,
                           int nbatch, int r, int C, int chunk_rows, int nchunks, OutT *dst, const int *skip,
                           DevStatus *st, cudaStream_t s, cudaError_t &err) {
  if (nrows % 32 || chunk_rows % 32 || C <= 8) return false;
  const int RT = r <= 16 ? 16 : (r <= 32 ? 32 : 64);
  const long long total = nrows * nbatch;
  CUtensorMap ma, mx;
  if (!make_tensor_map_f32(&ma, A, total, r, lda, 32, RT, true)) return false;
  if (!make_tensor_map_f32(&mx, X, total, C, ldx, 32, 64, true)) return false;
  const int nct = ceil_div(C, 64);
  if (RT == 16)
    err = reduce_tma_rt<16, OutT>(ma, mx, nrows, nbatch, r, C, chunk_rows, nchunks, nct, dst, skip, st, s);
  else if (RT == 32)
    err = reduce_tma_rt<32, OutT>(ma, mx, nrows, nbatch, r, C, chunk_rows, nchunks, nct, dst, skip, st, s);
  else
    err = reduce_tma_rt<64, OutT>(ma, mx, nrows, nbatch, r, C, chunk_rows, nchunks, nct, dst, skip, st, s);
  return true;
}

template <typename OutT>
__global__ void reduce_pass2_kernel(const double *__restrict__ partial, int nchunks, long long blk,
                                    OutT *out, const int *skip) {
  // 32 elements per CTA, the chunks split over 8 thread rows (row y sums
  // chunks y, y + 8, ...), the 8 row sums combined in a fixed order: the
  // long serial sums of the top levels (hundreds of chunks, few elements)
  // spread over 8x the threads and SMs.
  if (skip && *skip) return;
  __shared__ double part[8][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const long long e = (long long)blockIdx.x * 32 + tx;
  const int b = blockIdx.y;
  double acc = 0.0;
  if (e < blk) {
    const double *p = partial + (long long)b * nchunks * blk + e;
    for (int c = ty; c < nchunks; c += 8) acc += p[(long long)c * blk];
  }
  part[ty][tx] = acc;
  __syncthreads();
  if (ty == 0 && e < blk) {
    double sum = part[0][tx];
#pragma unroll
    for (int y = 1; y < 8; ++y) sum += part[y][tx];
    out[(long long)b * blk + e] = sum;
  }
}

// Row chunks per child so that about `target` CTAs run (at least 256 rows each).
static void reduce_plan(long long nrows, int nbatch, int C, int target, int &nchunks, int &chunk_rows) {
  const int nct = ceil_div(C, red_bn(C));
  const long long base = (long long)nct * nbatch;
  nchunks = 1;
  if (base < target)
    nchunks = (int)std::min<long long>(ceil_div(target, base), ceil_div(nrows, 256));
  nchunks = std::max(1, nchunks);
  // chunks of whole 64-row steps where the block allows (the tensor-core kernel stages 64 rows)
  const int step = nrows % 64 == 0 ? 64 : kRedBK;
  chunk_rows = (int)std::min<long long>(nrows, (long long)ceil_div(ceil_div(nrows, nchunks), step) * step);
  nchunks = ceil_div(nrows, chunk_rows);
}

// Sized for the largest split-K target the tuner may choose.
size_t reduce_workspace_doubles(long long nrows, int nbatch, int r, int C, int) {
  int nchunks, chunk_rows;
  reduce_plan(nrows, nbatch, C, kMaxRedCtasPerSm * kNumSMs, nchunks, chunk_rows);
  return nchunks > 1 ? (size_t)nbatch * nchunks * r * C : 0;
}

template <typename T, int RT, int BN, typename OutT>
static cudaError_t reduce_rt(const T *A, long long lda, const T *X, long long ldx, long long nrows, int nbatch,
                             int r, int C, int chunk_rows, int nchunks, int nct, OutT *dst, const int *skip,
                             cudaStream_t s) {
  const size_t bytes = sizeof(T) * ((size_t)kRedBK * (RT + 1) + (size_t)kRedBK * (BN + 1) + 4ull * RT * (BN + 1));
  auto k = reduce_tn_kernel<T, RT, BN, OutT>;
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
  }
  const long long nblk = (long long)nct * nchunks * nbatch;
  HODLR_LAUNCH(k, (unsigned)nblk, 256, bytes, s, A, lda, X, ldx, nrows, r, C, chunk_rows, nchunks, nct, dst, skip);
  return cudaGetLastError();
}

template <typename T, typename OutT>
static cudaError_t reduce_dispatch(const T *A, long long lda, const T *X, long long ldx, long long nrows,
                                   int nbatch, int r, int C, OutT *out, double *work, const int *skip,
                                   cudaStream_t s, DevStatus *st) {
  int nchunks, chunk_rows;
  reduce_plan(nrows, nbatch, C, current_tuning().red_ctas_per_sm * kNumSMs, nchunks, chunk_rows);
  const int bn = red_bn(C);
  const int nct = ceil_div(C, bn);
  cudaError_t e = cudaSuccess;
  // split-K partials are FP64 in the workspace; a single chunk writes the output type directly
  auto run = [&](auto *dst) -> cudaError_t {
    using D = typename std::remove_pointer<decltype(dst)>::type;
    bool done = false;
    cudaError_t err = cudaSuccess;
    if constexpr (sizeof(T) == 4) {
      done = reduce_tc_try<D>(A, lda, X, ldx, nrows, nbatch, r, C, chunk_rows, nchunks, dst, skip, st, s, err);
      if (!done)
        done = reduce_tma_try<D>(A, lda, X, ldx, nrows, nbatch, r, C, chunk_rows, nchunks, dst, skip, st, s, err);
    }
    if (done) return err;
#define HODLR_RED(RTV, BNV) \
  err = reduce_rt<T, RTV, BNV, D>(A, lda, X, ldx, nrows, nbatch, r, C, chunk_rows, nchunks, nct, dst, skip, s)
    if (bn == 8) {
      if (r <= 16) HODLR_RED(16, 8);
      else if (r <= 32) HODLR_RED(32, 8);
      else HODLR_RED(64, 8);
    } else {
      if (r <= 16) HODLR_RED(16, 64);
      else if (r <= 32) HODLR_RED(32, 64);
      else HODLR_RED(64, 64);
    }
#undef HODLR_RED
    return err;
  };
  if (nchunks > 1) {
    e = run(work);
    if (e != cudaSuccess) return e;
    const long long blk = (long long)r * C;
    dim3 grid(ceil_div(blk, 32), nbatch);
    HODLR_LAUNCH(reduce_pass2_kernel<OutT>, grid, 256, 0, s, work, nchunks, blk, out, skip);
  } else {
    e = run(out);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reduce_tn(const T *A, long long lda, const T *X, long long ldx, long long nrows,
                             int nbatch, int r, int C, double *out, double *work, const int *skip,
                             cudaStream_t s, DevStatus *st, float *out32) {
  if (C <= 0 || nbatch <= 0) return cudaSuccess;
  if (r < 1 || r > 64) return cudaErrorInvalidValue;
  if (out32) return reduce_dispatch<T, float>(A, lda, X, ldx, nrows, nbatch, r, C, out32, work, skip, s, st);
  return reduce_dispatch<T, double>(A, lda, X, ldx, nrows, nbatch, r, C, out, work, skip, s, st);
}

template cudaError_t launch_reduce_tn<double>(const double *, long long, const double *, long long, long long,
                                              int, int, int, double *, double *, const int *, cudaStream_t,
                                              DevStatus *, float *);
template cudaError_t launch_reduce_tn<float>(const float *, long long, const float *, long long, long long, int,
                                             int, int, double *, double *, const int *, cudaStream_t, DevStatus *,
                                             float *);

// ------------------------------------------------------------------ K5
// CTA tile 128 rows x 64 columns, K staged 32 at a time; each thread owns
// rows ti + 16a (a < 8) and columns 4tj .. 4tj+3 (coalesced read-modify-write
// of C along rows).
// The inner dimension is staged BK at a time: 32, or 8 for the rank-k outer
// products of the adjoint (K = nrhs <= 8).
static constexpr int kUpdBM = 128, kUpdBN = 64;

template <typename T, int BK>
__global__ void __launch_bounds__(256) update_nn_kernel(UpdateArgs a, int nrt, int nct) {
  if (a.skip && *a.skip) return;
  __shared__ __align__(16) T sA[BK][kUpdBM];
  __shared__ __align__(16) T sB[BK][kUpdBN + 1];  // +1: conflict-free column stores
  long long lin = blockIdx.x;
  const int rt = (int)(lin % nrt);
  lin /= nrt;
  const int ct = (int)(lin % nct);
  const int b = (int)(lin / nct);
  const int i0 = rt * kUpdBM, j0 = ct * kUpdBN;
  const T *A = reinterpret_cast<const T *>(a.A) + (long long)b * a.a_bstride;
  const double *B = a.B + (long long)(b >> 1) * a.b_s1 + (long long)((b & 1) ^ a.b_flip) * a.b_s2;
  T *C = reinterpret_cast<T *>(a.C) + (long long)b * a.c_bstride;
  const int tid = threadIdx.x, ti = tid & 15, tj = tid >> 4;
  T acc[8][4];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
  for (int q0 = 0; q0 < a.K; q0 += BK) {
    for (int e = tid; e < kUpdBM * BK; e += 256) {
      const int i = e % kUpdBM, q = e / kUpdBM;
      T v = T(0);
      if (i0 + i < a.M && q0 + q < a.K)
        v = a.a_trans ? A[(q0 + q) + (long long)(i0 + i) * a.lda] : A[i0 + i + (long long)(q0 + q) * a.lda];
      sA[q][i] = v;
    }
    for (int e = tid; e < BK * kUpdBN; e += 256) {
      const int q = e % BK, j = e / BK;
      double v = 0.0;
      if (q0 + q < a.K && j0 + j < a.N) {
        if (sizeof(T) == 4 && a.B32) {
          const float *B32 = a.B32 + (long long)(b >> 1) * a.b_s1 + (long long)((b & 1) ^ a.b_flip) * a.b_s2;
          v = a.b_trans ? B32[(j0 + j) + (long long)(q0 + q) * a.ldb] : B32[(q0 + q) + (long long)(j0 + j) * a.ldb];
        } else {
          v = a.b_trans ? B[(j0 + j) + (long long)(q0 + q) * a.ldb] : B[(q0 + q) + (long long)(j0 + j) * a.ldb];
          if (a.scale) v *= a.scale_cols ? a.scale[j0 + j] : a.scale[q0 + q];
        }
      }
      sB[q][j] = (T)v;
    }
    __syncthreads();
#pragma unroll 4
    for (int q = 0; q < BK; ++q) {
      T av[8], bv[4];
#pragma unroll
      for (int u = 0; u < 8; ++u) av[u] = sA[q][ti + 16 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) bv[v] = sB[q][tj * 4 + v];
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] += av[u] * bv[v];
    }
    __syncthreads();
  }
  const T alpha = (T)a.alpha;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int j = j0 + tj * 4 + v;
    if (j >= a.N) continue;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int i = i0 + ti + 16 * u;
      if (i < a.M) {
        T *c = C + i + (long long)j * a.ldc;
        *c = *c + alpha * acc[u][v];
      }
    }
  }
}

// K5, FP32, TMA: one CTA per (BM-row x 64-column) tile of a block.  Thread 0
// issues the A tile (BM rows x KMAX ranks) and the C tile (BM x 64) as 2-D
// TMA loads on two mbarriers; meanwhile all threads stage op(B_b) (FP64 eta,
// scaled, rounded to FP32) into shared memory.  Each thread owns float4 runs
// of rows (4 tr + 64 g) and 4 columns; the product is added to the C tile in
// shared memory, which thread 0 writes back with one TMA store (rows and
// columns beyond the tensor are clipped by the copy engine).
// Preconditions (host-checked): A not transposed, blocks of exactly M rows at
// stride M in A and C, M a multiple of BM, K <= KMAX, 16-byte alignment.
template <int BM, int KMAX>
__global__ void __launch_bounds__(256)
update_tma_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapC, UpdateArgs a,
                  int nrt, int nct, DevStatus *st) {
  if (a.skip && *a.skip) return;
  constexpr int BN = 64, RG = BM / 64;
  extern __shared__ unsigned char smem_raw[];
  float *base = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                          ~static_cast<uintptr_t>(127));
  float *sC = base;                 // [BN][BM]
  float *sA = sC + BN * BM;         // [KMAX][BM]
  float *sB = sA + KMAX * BM;       // [KMAX][BN]
  __shared__ __align__(8) uint64_t bars[2];
  long long lin = blockIdx.x;
  const int rt = (int)(lin % nrt);
  lin /= nrt;
  const int ct = (int)(lin % nct);
  const int b = (int)(lin / nct);
  const int i0 = rt * BM, j0 = ct * BN;
  const long long rowA = (long long)b * a.a_bstride + i0, rowC = (long long)b * a.c_bstride + i0;
  const int tid = threadIdx.x, tr = tid & 15, tc = tid >> 4;
  if (tid == 0) {
    prefetch_tensormap(&mapA);
    prefetch_tensormap(&mapC);
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(&bars[0], KMAX * BM * 4);
    tma_load_2d(sA, &mapA, &bars[0], (int)rowA, 0);
    mbar_arrive_expect_tx(&bars[1], BN * BM * 4);
    tma_load_2d(sC, &mapC, &bars[1], (int)rowC, j0);
  }
  const long long boff = (long long)(b >> 1) * a.b_s1 + (long long)((b & 1) ^ a.b_flip) * a.b_s2;
  if (a.B32) {
    const float *B = a.B32 + boff;
    constexpr int PER = KMAX * BN / 256;
    float x[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = tid + 256 * u, q = e / BN, j = e % BN;
      x[u] = (q < a.K && j0 + j < a.N)
                 ? (a.b_trans ? B[(j0 + j) + (long long)q * a.ldb] : B[q + (long long)(j0 + j) * a.ldb])
                 : 0.f;
    }
#pragma unroll
    for (int u = 0; u < PER; ++u) sB[tid + 256 * u] = x[u];
  } else {
    const double *B = a.B + boff;
    // all of this thread's eta loads in flight at once, then convert and store
    constexpr int PER = KMAX * BN / 256;
    double x[PER], sc[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = tid + 256 * u, q = e / BN, j = e % BN;
      const bool in = q < a.K && j0 + j < a.N;
      x[u] = in ? (a.b_trans ? B[(j0 + j) + (long long)q * a.ldb] : B[q + (long long)(j0 + j) * a.ldb]) : 0.0;
      sc[u] = (in && a.scale) ? (a.scale_cols ? a.scale[j0 + j] : a.scale[q]) : 1.0;
    }
#pragma unroll
    for (int u = 0; u < PER; ++u) sB[tid + 256 * u] = (float)(x[u] * sc[u]);
  }
  bool ok = mbar_wait_bounded(&bars[0], 0);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) {
      report_error(st, HODLR_ERR_TIMEOUT, blockIdx.x);
      (void)mbar_wait_bounded(&bars[1], 0);
    }
    return;
  }
  float acc[RG * 4][4];
#pragma unroll
  for (int u = 0; u < RG * 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
#pragma unroll 4
  for (int q = 0; q < a.K; ++q) {
    const float4 bv = *reinterpret_cast<const float4 *>(sB + q * BN + 4 * tc);
#pragma unroll
    for (int g = 0; g < RG; ++g) {
      const float4 av = *reinterpret_cast<const float4 *>(sA + q * BM + 64 * g + 4 * tr);
      const float ar[4] = {av.x, av.y, av.z, av.w}, br[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) acc[g * 4 + ii][jj] = fmaf(ar[ii], br[jj], acc[g * 4 + ii][jj]);
    }
  }
  ok = mbar_wait_bounded(&bars[1], 0);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) report_error(st, HODLR_ERR_TIMEOUT, blockIdx.x);
    return;
  }
  const float alpha = (float)a.alpha;
#pragma unroll
  for (int jj = 0; jj < 4; ++jj)
#pragma unroll
    for (int g = 0; g < RG; ++g) {
      float4 *c = reinterpret_cast<float4 *>(sC + (4 * tc + jj) * BM + 64 * g + 4 * tr);
      float4 v = *c;
      v.x = fmaf(alpha, acc[g * 4 + 0][jj], v.x);
      v.y = fmaf(alpha, acc[g * 4 + 1][jj], v.y);
      v.z = fmaf(alpha, acc[g * 4 + 2][jj], v.z);
      v.w = fmaf(alpha, acc[g * 4 + 3][jj], v.w);
      *c = v;
    }
  fence_proxy_async_smem();
  __syncthreads();
  if (tid == 0) {
    tma_store_2d(&mapC, sC, (int)rowC, j0);
    tma_store_commit();
    tma_store_wait_read_all();
  }
}

template <int BM, int KMAX>
static cudaError_t update_tma_launch(const CUtensorMap &ma, const CUtensorMap &mc, const UpdateArgs &a, int nrt,
                                     int nct, DevStatus *st, cudaStream_t s) {
  const size_t bytes = sizeof(float) * ((size_t)64 * BM + (size_t)KMAX * BM + (size_t)KMAX * 64) + 128;
  auto k = update_tma_kernel<BM, KMAX>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long long nblk = (long long)nrt * nct * a.nbatch;
  HODLR_LAUNCH(k, (unsigned)nblk, 256, bytes, s, ma, mc, a, nrt, nct, st);
  return cudaGetLastError();
}

static bool update_tma_try(const UpdateArgs &a, DevStatus *st, cudaStream_t s, cudaError_t &err) {
  if (a.a_trans || a.K < 1 || a.K > 64 || a.a_bstride != a.M || a.c_bstride != a.M) return false;
  const int want = current_tuning().upd_bm;
  int BM = a.M % 128 == 0 ? 128 : (a.M % 64 == 0 ? 64 : 0);
  if (want == 64 && a.M % 64 == 0) BM = 64;
  if (!BM) return false;
  const int KMAX = a.K <= 32 ? 32 : 64;
  const long long rows = (long long)a.M * a.nbatch;
  CUtensorMap ma, mc;
  if (!make_tensor_map_f32(&ma, static_cast<const float *>(a.A), rows, a.K, a.lda, BM, KMAX, false)) return false;
  if (!make_tensor_map_f32(&mc, static_cast<const float *>(a.C), rows, a.N, a.ldc, BM, 64, false)) return false;
  const int nrt = a.M / BM, nct = ceil_div(a.N, 64);
  if (BM == 128)
    err = KMAX == 32 ? update_tma_launch<128, 32>(ma, mc, a, nrt, nct, st, s)
                     : update_tma_launch<128, 64>(ma, mc, a, nrt, nct, st, s);
  else
    err = KMAX == 32 ? update_tma_launch<64, 32>(ma, mc, a, nrt, nct, st, s)
                     : update_tma_launch<64, 64>(ma, mc, a, nrt, nct, st, s);
  return true;
}

// update_tc.cu: the tcgen05 path (FP32 operands split into bf16 planes)
bool update_tc_try(const UpdateArgs &a, DevStatus *st, cudaStream_t s, cudaError_t &err);

template <typename T>
cudaError_t launch_update_nn(const UpdateArgs &a, cudaStream_t s, DevStatus *st) {
  if (a.M <= 0 || a.N <= 0 || a.nbatch <= 0) return cudaSuccess;
  if constexpr (sizeof(T) == 4) {
    cudaError_t e = cudaSuccess;
    if (update_tc_try(a, st, s, e)) return e;
    if (update_tma_try(a, st, s, e)) return e;
  }
  const int nrt = ceil_div(a.M, kUpdBM), nct = ceil_div(a.N, kUpdBN);
  const long long nblk = (long long)nrt * nct * a.nbatch;
  if (a.K <= 8)
    HODLR_LAUNCH((update_nn_kernel<T, 8>), (unsigned)nblk, 256, 0, s, a, nrt, nct);
  else
    HODLR_LAUNCH((update_nn_kernel<T, 32>), (unsigned)nblk, 256, 0, s, a, nrt, nct);
  return cudaGetLastError();
}
template cudaError_t launch_update_nn<double>(const UpdateArgs &, cudaStream_t, DevStatus *);
template cudaError_t launch_update_nn<float>(const UpdateArgs &, cudaStream_t, DevStatus *);

}  // namespace hodlr

extern "C" int hodlr_debug_wait_fault(int cta, int stage, long long budget_cycles) {
  if (cta < -1 || (cta >= 0 && stage < 0) || budget_cycles < 0 || budget_cycles > 1000000000LL)
    return hodlr::set_last_error(HODLR_ERR_INVALID_ARG, "debug_wait_fault: bad arguments");
  const hodlr::WaitFault wf = {cta, cta < 0 ? -1 : stage, cta < 0 ? 0 : budget_cycles};
  cudaError_t e = cudaMemcpyToSymbol(hodlr::g_wait_fault, &wf, sizeof wf);
  if (e == cudaSuccess) e = hodlr::reduce_tc_set_wait_fault(wf);
  if (e != cudaSuccess) return hodlr::set_last_error(HODLR_ERR_CUDA, cudaGetErrorString(e));
  return HODLR_OK;
}
