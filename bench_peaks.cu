// Benchmark helper (not part of the solver library): the FP32 and FP64 FMA
// issue rates and the warp-level bf16 MMA rate of the current GPU, the
// denominators bench.py uses for the roofline fractions of the CUDA-core
// kernels (the FP32 GEMMs on the FMA pipe, the FP64 capacitance
// factorisation on the FP64 pipe).  Each thread runs eight independent
// chains; every index is the thread's own output slot.  Built by bench.py
// (build_peak_probe) into bench_peaks.so next to this file.
#include <cuda_runtime.h>

namespace probe {

template <typename T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T *out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
    x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
static cudaError_t time_chain(int iters, double *tflops) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int threads = 256, blocks = sms * 8;
  T *out = nullptr;
  e = cudaMalloc(&out, sizeof(T) * threads * blocks);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 3; ++rep) {  // the first run loads the module
    cudaEventRecord(e0, 0);
    fma_chain_kernel<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1, 0);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return e;
  *tflops = 2.0 * 8.0 * iters * (double)threads * blocks / (best * 1e-3) / 1e12;
  return cudaSuccess;
}

// Warp-level bf16 MMA (m16n8k16, FP32 accumulate) issue rate: eight
// independent accumulator tiles per warp, register operands only.
__global__ void __launch_bounds__(256) mma_chain_kernel(float *out, int iters) {
  const unsigned a0 = 0x3f803f80u + threadIdx.x, a1 = a0 ^ 1u, a2 = a0 ^ 2u, a3 = a0 ^ 3u;
  const unsigned b0 = 0x3f003f00u + threadIdx.x, b1 = b0 ^ 1u;
  float c[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) c[j][q] = 0.f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
          "{%0,%1,%2,%3};\n"
          : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += c[j][0] + c[j][1] + c[j][2] + c[j][3];
  out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

static cudaError_t time_mma(int iters, double *tflops) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int threads = 256, blocks = sms * 4;
  float *out = nullptr;
  e = cudaMalloc(&out, sizeof(float) * threads * blocks);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0, 0);
    mma_chain_kernel<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1, 0);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return e;
  *tflops = 2.0 * 16 * 8 * 16 * 8.0 * iters * (double)(threads / 32) * blocks / (best * 1e-3) / 1e12;
  return cudaSuccess;
}

}  // namespace probe

// Both return 0 or the CUDA error code.
extern "C" __attribute__((visibility("default"))) int bench_probe_mma_bf16(double *tflops) {
  if (!tflops) return (int)cudaErrorInvalidValue;
  return (int)probe::time_mma(4096, tflops);
}

extern "C" __attribute__((visibility("default"))) int bench_probe_fp_peaks(double *ffma_tflops,
                                                                           double *dfma_tflops) {
  if (!ffma_tflops || !dfma_tflops) return (int)cudaErrorInvalidValue;
  cudaError_t e = probe::time_chain<float>(65536, ffma_tflops);
  if (e == cudaSuccess) e = probe::time_chain<double>(4096, dfma_tflops);
  return (int)e;
}
