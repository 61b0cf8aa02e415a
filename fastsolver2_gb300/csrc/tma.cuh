// Tensor-memory-accelerator (TMA) helpers for sm_103a: 2-D tiled bulk
// copies global -> shared (cp.async.bulk.tensor) completing on an mbarrier,
// bounded mbarrier waits, and host-side tensor-map encoding through the
// driver entry point (no link against libcuda).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "common.cuh"

namespace hodlr {

// ------------------------------------------------------------------ device
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for phase `parity` of an mbarrier for at most ~max_cycles SM clocks
// (about half a second at GB300 clocks); false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity,
                                                  long long max_cycles = 1000000000LL) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > max_cycles) return false;
  return true;
}

// 2-D tile load: box at (x = innermost coordinate, y) into shared memory,
// completion counted in bytes on `bar`.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// 3-D tile load: box at (x = innermost, y, z) into shared memory, completion
// counted in bytes on `bar`.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// 2-D tile store shared -> global, tracked by the bulk async-group of the
// issuing thread.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, const void *src, int x, int y) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];"
               ::"l"(map), "r"(x), "r"(y), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void tma_store_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Wait until every committed store has finished reading its shared memory
// (the global writes complete on their own; the CTA may then exit).
__device__ __forceinline__ void tma_store_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// Wait until every committed store has finished reading shared memory and
// its writes are performed.
__device__ __forceinline__ void tma_store_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// Order this thread's generic-proxy shared-memory writes before later async-proxy reads.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

// Byte offset of 16-byte chunk `chunk` of row `row` in a tile written with
// CU_TENSOR_MAP_SWIZZLE_128B (rows of 128 bytes, tile base 1024-byte aligned).
__device__ __forceinline__ int swz128(int row, int chunk) { return row * 128 + ((chunk ^ (row & 7)) << 4); }

// ------------------------------------------------------------------- host
// 2-D tensor map over a column-major FP32 matrix: `rows` x `cols`, leading
// dimension `ld` (elements), box `box_rows` x `box_cols`.  Out-of-range
// elements load as zero.  Returns false if the driver refuses it (the
// caller then takes its non-TMA path).
bool make_tensor_map_f32(CUtensorMap *map, const float *base, long long rows, long long cols, long long ld,
                         int box_rows, int box_cols, bool swizzle128);
// The same over a column-major FP64 matrix, no swizzle.
bool make_tensor_map_f64(CUtensorMap *map, const double *base, long long rows, long long cols, long long ld,
                         int box_rows, int box_cols);
// 3-D tensor map over the same column-major FP32 matrix seen as 32-row
// blocks: (32 rows, rows / 32 blocks, cols), box (32, row_blocks, box_cols)
// with the 128-byte swizzle -- a box of 32 * row_blocks rows whose 128-byte
// lines (one 32-row block of one column) are swizzled as 2-D boxes of 32
// rows are.  rows must be a multiple of 32.
bool make_tensor_map_f32_rowblocks(CUtensorMap *map, const float *base, long long rows, long long cols, long long ld,
                                   int row_blocks, int box_cols);
// 2-D tensor map over a bf16 matrix stored with `inner` contiguous elements
// per line (line pitch `ld` elements, `outer` lines); box box_inner x
// box_outer, swizzle 0, 32, 64 or 128 bytes.  Out-of-range elements load as
// zero.
bool make_tensor_map_bf16(CUtensorMap *map, const void *base, long long inner, long long outer, long long ld,
                          int box_inner, int box_outer, int swizzle_bytes);

}  // namespace hodlr
