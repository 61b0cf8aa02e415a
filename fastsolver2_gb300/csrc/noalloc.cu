// hodlr_gemm_reduce_noalloc: the per-partition reduction W_p = V_p^T U_p of
// hodlr_gemm_reduce, for callers that are not allowed to allocate device
// memory.
//
// Who cannot allocate: callers whose framework owns the whole device through
// its own caching allocator and forbids side allocations, and latency-critical
// loops that cannot afford the implicit device-wide synchronisation
// cudaMalloc / cudaFree can cause.  hodlr_gemm_reduce needs scratch for its
// split-K partial sums and per-partition blocks and takes it with cudaMalloc;
// this variant takes the same scratch from one fixed device array instead.
// It runs on the legacy default stream and synchronises with it before it
// returns, so it is a call for ordinary (uncaptured) host code.
//
// The scratch is a file-scope __device__ array of kNoAllocDoubles doubles
// (16 MiB): every GPU that loads this library holds it until the process
// exits.  Host code cannot use the array's name as a device address (on the
// host it names a host-side shadow), so the first call on each device looks
// the address up with cudaGetSymbolAddress while that device is current and
// caches it.  cudaDeviceReset unloads the library's device code, which makes
// the cached address stale: a process that resets a device must not call this
// function on that device afterwards.  Every call on a device shares the one
// array: calls whose work overlaps on the GPU (concurrent streams, other host
// threads) race on it.  The kernels write every scratch entry they later read
// (partial sums and blocks are stored, never accumulated), so the contents
// left by a previous call need no clearing.  Sizes whose scratch would exceed
// the array are rejected with HODLR_ERR_INVALID_ARG.
#include <mutex>

#include "kernels.cuh"

namespace hodlr {

static constexpr size_t kNoAllocDoubles = size_t(1) << 21;  // 16 MiB of FP64 scratch
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

static constexpr int kMaxDevices = 64;
static double *g_scratch_addr[kMaxDevices] = {};
static std::mutex g_scratch_mu;

// Device address of g_noalloc_scratch on the current device (looked up once
// per device, with that device current).
static int scratch_address(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_last_error(HODLR_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_last_error(HODLR_ERR_INVALID_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_last_error(HODLR_ERR_CUDA, e != cudaSuccess ? cudaGetErrorString(e) : "null symbol address");
    g_scratch_addr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_addr[dev];
  return HODLR_OK;
}

}  // namespace hodlr

using namespace hodlr;

extern "C" int hodlr_gemm_reduce_noalloc(int nrow, int nPart, int ncolV, int ncolU, const double *V, int64_t ldv,
                                         const double *U, int64_t ldu, double *W, int64_t ldw) {
  if (!V || !U || !W || nPart < 1 || nrow % nPart || ncolV < 1 || ncolV > 64 || ncolU < 1 || ldv < nrow ||
      ldu < nrow || ldw < (int64_t)nPart * ncolV)
    return set_last_error(HODLR_ERR_INVALID_ARG, "gemm_reduce_noalloc: bad arguments");
  const long long rows = nrow / nPart;
  const size_t blocks = (size_t)nPart * ncolV * ncolU;
  const size_t work = reduce_workspace_doubles(rows, nPart, ncolV, ncolU, 8);
  if (blocks + work > kNoAllocDoubles)
    return set_last_error(HODLR_ERR_INVALID_ARG,
                          "gemm_reduce_noalloc: nPart*ncolV*ncolU plus the split-K partial sums exceed the "
                          "fixed scratch of 2097152 doubles (16 MiB); use hodlr_gemm_reduce");
  double *scratch = nullptr;
  int st = scratch_address(&scratch);
  if (st != HODLR_OK) return st;
  double *out = scratch;            // per-partition blocks, ncolV x ncolU each
  double *partial = scratch + blocks;  // split-K partial sums (written before read)
  cudaError_t e = launch_reduce_tn<double>(V, ldv, U, ldu, rows, nPart, ncolV, ncolU, out, partial, nullptr, 0);
  if (e != cudaSuccess) return set_last_error(HODLR_ERR_CUDA, cudaGetErrorString(e));
  for (int p = 0; p < nPart; ++p) {  // block p -> rows p*ncolV of W (a copy, not an allocation)
    e = cudaMemcpy2DAsync(W + (long long)p * ncolV, sizeof(double) * ldw, out + (size_t)p * ncolV * ncolU,
                          sizeof(double) * ncolV, sizeof(double) * ncolV, ncolU, cudaMemcpyDeviceToDevice, 0);
    if (e != cudaSuccess) return set_last_error(HODLR_ERR_CUDA, cudaGetErrorString(e));
  }
  e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) return set_last_error(HODLR_ERR_CUDA, cudaGetErrorString(e));
  return HODLR_OK;
}
