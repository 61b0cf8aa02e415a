// Shared definitions of the GB300 HODLR kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "hodlr_gb300.h"

namespace hodlr {

// Device-side status block of a handle: the first error wins.
struct DevStatus {
  int code;
  int pad;
  long long index;
  int done;       // refinement converged flag (predicates correction kernels)
  int iters;      // corrections applied
  double resid;   // last relative residual
};

__device__ __forceinline__ void report_error(DevStatus *st, int code, long long index) {
  if (st && atomicCAS(&st->code, 0, code) == 0) st->index = index;
}

template <typename T> __device__ __forceinline__ T dabs(T x) { return x < T(0) ? -x : x; }

// FP64 -> FP32, round to nearest even, on the integer pipes.  GB300 runs
// FP64 instructions -- the double -> float conversion among them -- at a
// small fraction of the FP32 rate, so kernels that turn FP64 data into FP32
// were paced by the conversion.  For magnitudes in the FP32 normal range
// (double exponent 897 .. 1150) the float is the double's sign, its exponent
// rebased from 1023 to 127 and the top 23 of its 52 fraction bits, rounded on
// the 29 bits dropped with ties to even; a carry out of the fraction moves
// into the exponent, up to infinity past the largest float, as the rounding
// rule asks.  Zeros keep their sign; results in the subnormal range,
// infinities and NaNs take the hardware conversion.
__device__ __forceinline__ float f64_to_f32_rn(double d) {
  const unsigned hi = static_cast<unsigned>(__double2hiint(d)), lo = static_cast<unsigned>(__double2loint(d));
  const unsigned ahi = hi & 0x7FFFFFFFu;
  if (ahi - (897u << 20) < ((1151u - 897u) << 20)) {
    // (e << 23 | fraction) mod 2^32, less (896 << 23) mod 2^32 = 0xC0000000
    const unsigned bits = __funnelshift_l(lo, ahi, 3) - 0xC0000000u;
    const unsigned up = ((lo & 0x1FFFFFFFu) + 0x0FFFFFFFu + (bits & 1u)) >> 29;
    return __uint_as_float((bits + up) | (hi & 0x80000000u));
  }
  if ((ahi | lo) == 0) return __uint_as_float(hi);
  return __double2float_rn(d);
}

// Host-side launch accounting (every kernel launch of the library goes
// through HODLR_LAUNCH so hodlr_kernel_launches() can report it).
void count_launch();
// HODLR_DEBUG_SYNC=1 in the environment: synchronise after every launch
// (outside graph capture) and print the first failing kernel's name.
bool debug_sync();
void debug_after_launch(const char *name, cudaStream_t s);

#define HODLR_LAUNCH(kernel, grid, block, smem, stream, ...)                 \
  do {                                                                       \
    ::hodlr::count_launch();                                                 \
    (void)cudaGetLastError(); /* report this launch's own error only */      \
    kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);              \
    if (::hodlr::debug_sync()) ::hodlr::debug_after_launch(#kernel, stream); \
  } while (0)

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Lets `func` (a __global__ function) take up to the device's opt-in shared
// memory per block, less its static shared memory.  The attribute is only an
// upper bound -- each launch's own size decides occupancy -- so it is raised
// once per (function, device) and never lowered: a graph captured with a
// large launch stays launchable after the same kernel ran with a smaller size.
cudaError_t allow_max_dyn_smem(const void *func);
template <typename K> inline cudaError_t allow_dyn_smem(K kernel, size_t bytes) {
  return bytes <= 48 * 1024 ? cudaSuccess : allow_max_dyn_smem(reinterpret_cast<const void *>(kernel));
}

// Launch shape of an n x c column-major elementwise pass: blockIdx.y strides
// over columns, x over rows (no 64-bit index division in the kernels).
inline dim3 grid2d(long long n, int c) {
  const int y = c < 1 ? 1 : (c > 65535 ? 65535 : c);
  long long x = (n + 255) / 256;
  const long long cap = 4864 / y > 0 ? 4864 / y : 1;
  if (x > cap) x = cap;
  if (x < 1) x = 1;
  return dim3((unsigned)x, (unsigned)y);
}

#define HODLR_FOR_2D(i, j, n, c)                                                     \
  for (long long j = blockIdx.y; j < (long long)(c); j += gridDim.y)                \
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (n);    \
         i += (long long)gridDim.x * blockDim.x)

}  // namespace hodlr
