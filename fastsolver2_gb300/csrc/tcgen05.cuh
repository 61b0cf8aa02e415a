// tcgen05 (5th-generation tensor core) primitives for sm_103a, as inline
// PTX: tensor-memory allocation, single-thread MMA issue with completion on
// an mbarrier, tensor-memory loads, the thread-sync fences, and the
// shared-memory matrix descriptor of the K-major 64-byte-swizzled layout
// that a TMA load with CU_TENSOR_MAP_SWIZZLE_64B produces.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "tma.cuh"

namespace hodlr {

// kind::f16 instruction descriptor: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr unsigned tc_idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) | ((unsigned)(m >> 4) << 24);
}

// Shared-memory matrix descriptor: K-major, 64-byte swizzle (rows of 64
// bytes, 8-row atoms of 512 bytes = stride-dimension offset), version 1.
__device__ __forceinline__ uint64_t desc_sw64(unsigned saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

// The same with the 128-byte swizzle (rows of 128 bytes = 64 bf16, 8-row
// atoms of 1024 bytes).
__device__ __forceinline__ uint64_t desc_sw128(unsigned saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void tc_alloc(unsigned *dst, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_mma(unsigned d, uint64_t a, uint64_t b, unsigned idesc, unsigned accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The same with A read from tensor memory: row i of A in lane i, two bf16
// per 32-bit column (the lower K index in the low half), K 16 = 8 columns
// from column `a` on.
__device__ __forceinline__ void tc_mma_ta(unsigned d, unsigned a, uint64_t b, unsigned idesc, unsigned accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
      "r"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The barrier receives one arrival when every tcgen05.mma this thread issued has completed.
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_ld32(unsigned taddr, unsigned (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_ld16(unsigned taddr, unsigned (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_ld4(unsigned taddr, unsigned (&v)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
               : "r"(taddr));
}
// Each thread of the warp writes 4 consecutive columns of its lane (the
// warp's quarter of the lanes); tc_wait_st makes the writes complete.
__device__ __forceinline__ void tc_st4(unsigned taddr, const uint4 &v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr), "r"(v.x), "r"(v.y),
               "r"(v.z), "r"(v.w)
               : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// Waits for this thread's tensor-memory loads; the registers pass through
// so that no use of them is scheduled before the wait.
template <int N, int W>
__device__ __forceinline__ void tc_wait_ld(unsigned (&v)[N][W]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int a = 0; a < N; ++a)
#pragma unroll
    for (int b = 0; b < W; ++b) asm volatile("" : "+r"(v[a][b]));
}

// Plain arrival on an mbarrier (warp-role kernels: one per thread of a role).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded wait of a warp-role kernel: false once the wait ran past `limit`
// SM clocks (it then sets *abort) or another role set *abort, so that every
// role leaves its loop when one of them gave up.
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t *bar, unsigned parity, int *abort, long long limit) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*(volatile int *)abort) return false;
    if (clock64() - t0 > limit) {
      *(volatile int *)abort = 1;
      return false;
    }
  }
  return true;
}

// Exact three-way bf16 split of two FP32 values, x = h + m + l (24
// significant bits; both subtractions are exact), for FP32-class products on
// the bf16 tensor cores from the six partial products down to 2^-16.  Each
// plane's pair is one packed conversion (value a in the low half, the lower
// address); widening a bf16 back to FP32 is exact.
__device__ __forceinline__ void split3_pair(float a, float b, unsigned &h, unsigned &m, unsigned &l) {
  const __nv_bfloat162 hb = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(hb);
  const float ra = a - hf.x, rb = b - hf.y;
  const __nv_bfloat162 mb = __floats2bfloat162_rn(ra, rb);
  const float2 mf = __bfloat1622float2(mb);
  const __nv_bfloat162 lb = __floats2bfloat162_rn(ra - mf.x, rb - mf.y);
  h = *reinterpret_cast<const unsigned *>(&hb);
  m = *reinterpret_cast<const unsigned *>(&mb);
  l = *reinterpret_cast<const unsigned *>(&lb);
}

// Byte offset of 16-byte chunk c (of 4) of row i in a K-major tile of 64-byte
// rows with the 64-byte swizzle (chunk index XOR address bits 7-8; the tile
// base is 1024-byte aligned).
__device__ __forceinline__ int swz64(int i, int c) { return i * 64 + ((c ^ ((i >> 1) & 3)) << 4); }

// Writes the three planes of 8 consecutive K values of one row (16 bytes
// of each plane).
__device__ __forceinline__ void put_planes(unsigned char *p0, int plane_bytes, int off, const float (&x)[8]) {
  uint4 h, m, l;
  split3_pair(x[0], x[1], h.x, m.x, l.x);
  split3_pair(x[2], x[3], h.y, m.y, l.y);
  split3_pair(x[4], x[5], h.z, m.z, l.z);
  split3_pair(x[6], x[7], h.w, m.w, l.w);
  *reinterpret_cast<uint4 *>(p0 + off) = h;
  *reinterpret_cast<uint4 *>(p0 + plane_bytes + off) = m;
  *reinterpret_cast<uint4 *>(p0 + 2 * plane_bytes + off) = l;
}

// The same for 4 consecutive K values (8 bytes of each plane).
__device__ __forceinline__ void put_planes4(unsigned char *p0, int plane_bytes, int off, const float4 &v) {
  uint2 h, m, l;
  split3_pair(v.x, v.y, h.x, m.x, l.x);
  split3_pair(v.z, v.w, h.y, m.y, l.y);
  *reinterpret_cast<uint2 *>(p0 + off) = h;
  *reinterpret_cast<uint2 *>(p0 + plane_bytes + off) = m;
  *reinterpret_cast<uint2 *>(p0 + 2 * plane_bytes + off) = l;
}

}  // namespace hodlr
