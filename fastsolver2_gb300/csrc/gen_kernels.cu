// Seeded synthetic problem generator (device side).
//
// fastSolver2 generates its inputs from per-partition seeds on the CPU
// (InitMatrixTask src/tasks/init_matrix.cc:35-73, DenseBlockTask
// src/tasks/dense_block.cc:35-76).  For the large configurations the inputs
// are generated where they are used, in HBM: a counter-based generator
// (splitmix64 hashing of (seed, stream, index), Box-Muller) so that any
// element is a pure function of its coordinates and launches parallelise
// freely.
#include <algorithm>

#include "kernels.cuh"

namespace hodlr {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double gauss(unsigned long long seed, unsigned long long stream,
                                        unsigned long long idx) {
  const unsigned long long h1 = mix64(seed ^ mix64(stream * 0xD1B54A32D192ED03ull + idx));
  const unsigned long long h2 = mix64(h1 ^ 0x5851F42D4C957F2Dull);
  const double u1 = ((double)(h1 >> 11) + 1.0) * 0x1.0p-53;  // (0, 1]
  const double u2 = (double)(h2 >> 11) * 0x1.0p-53;          // [0, 1)
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

__global__ void gaussian_kernel(double *X, long long ld, long long n, int c, unsigned long long seed,
                                unsigned long long stream, double scale) {
  HODLR_FOR_2D(i, j, n, c) X[i + j * ld] = scale * gauss(seed, stream, (unsigned long long)(i + j * n));
}

cudaError_t launch_gaussian(double *X, long long ld, long long n, int c, unsigned long long seed,
                            unsigned long long stream, double scale, cudaStream_t s) {
  const long long total = n * c;
  if (total == 0) return cudaSuccess;
  const int grid = (int)std::min<long long>(ceil_div(total, 256), 152 * 32);
  HODLR_LAUNCH(gaussian_kernel, grid, 256, 0, s, X, ld, n, c, seed, stream, scale);
  return cudaGetLastError();
}

__global__ void gen_leaves_kernel(double *D, int m, long long total, unsigned long long seed, double shift) {
  const double sc = 1.0 / sqrt((double)m);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long w = e % ((long long)m * m);
    const int i = (int)(w % m), j = (int)(w / m);
    D[e] = sc * gauss(seed, 0x1EAFull, (unsigned long long)e) + (i == j ? shift : 0.0);
  }
}

cudaError_t launch_gen_leaves(double *D, int m, int nleaf, unsigned long long seed, double shift,
                              cudaStream_t s) {
  const long long total = (long long)nleaf * m * m;
  const int grid = (int)std::min<long long>(ceil_div(total, 256), 152 * 32);
  HODLR_LAUNCH(gen_leaves_kernel, grid, 256, 0, s, D, m, total, seed, shift);
  return cudaGetLastError();
}

// One CTA per Gram matrix: Cholesky G = R^T R in shared memory, then Rinv.
__global__ void chol_inv_kernel(const double *G, double *Rinv, int r, DevStatus *st) {
  extern __shared__ double sm[];
  double *R = sm;          // r x r, upper
  double *Q = sm + r * r;  // r x r, Rinv
  const int b = blockIdx.x;
  const double *g = G + (long long)b * r * r;
  for (int e = threadIdx.x; e < r * r; e += blockDim.x) {
    R[e] = g[e];
    Q[e] = 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    bool ok = true;
    for (int j = 0; j < r && ok; ++j) {
      double d = R[j + j * r];
      for (int k = 0; k < j; ++k) d -= R[k + j * r] * R[k + j * r];
      if (!(d > 0.0)) {
        ok = false;
        break;
      }
      d = sqrt(d);
      R[j + j * r] = d;
      for (int c = j + 1; c < r; ++c) {
        double v = R[j + c * r];
        for (int k = 0; k < j; ++k) v -= R[k + j * r] * R[k + c * r];
        R[j + c * r] = v / d;
      }
    }
    if (!ok) {
      report_error(st, HODLR_ERR_SINGULAR_CAPACITANCE, b);
    } else {
      // Rinv: solve R Q = I column by column (upper triangular back substitution)
      for (int c = 0; c < r; ++c)
        for (int i = c; i >= 0; --i) {
          double v = (i == c) ? 1.0 : 0.0;
          for (int k = i + 1; k <= c; ++k) v -= R[i + k * r] * Q[k + c * r];
          Q[i + c * r] = v / R[i + i * r];
        }
    }
  }
  __syncthreads();
  double *o = Rinv + (long long)b * r * r;
  for (int e = threadIdx.x; e < r * r; e += blockDim.x) o[e] = Q[e];
}

cudaError_t launch_chol_inv(const double *G, double *Rinv, int r, int nbatch, DevStatus *st, cudaStream_t s) {
  const size_t bytes = (size_t)2 * r * r * sizeof(double);
  cudaError_t e = allow_dyn_smem(chol_inv_kernel, bytes);
  if (e != cudaSuccess) return e;
  HODLR_LAUNCH(chol_inv_kernel, nbatch, 64, bytes, s, G, Rinv, r, st);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The reference's own seeded generator, bit for bit.  PtrMatrix::rand(seed,
// offset) (src/ptr_matrix.cc:62-71) fills a block of a partitioned matrix in
// row-major order from one drand48 stream per partition (Matrix::rand,
// src/matrix.cc:250-297; the per-partition seeds travel in the MapSeed
// argument maps, src/lmatrix.cc:327-360).  drand48 is the POSIX 48-bit
// linear congruential generator X' = (a X + c) mod 2^48, a = 0x5DEECE66D,
// c = 0xB, seeded as X0 = (seed mod 2^32) 2^16 + 0x330E; a draw returns the
// new state times 2^-48 (exact in FP64) and lrand48 its top 31 bits.  A row
// reaches its first state by jumping ahead -- the affine map raised to the
// row's draw index by binary powering -- so rows fill in parallel.

__global__ void rand_block_kernel(const long long *seeds, int npart, long long rows, int cols, double offset,
                                  double *A, long long lda) {
  const long long total = (long long)npart * rows;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long k = e / rows, i = e % rows;
    unsigned long long x = lcg_jump(lcg_seed(seeds[k]), (unsigned long long)i * (unsigned long long)cols);
    double *a = A + k * rows + i;
    for (int j = 0; j < cols; ++j) {
      x = lcg_step(x);
      a[(long long)j * lda] = __dadd_rn((double)x * 0x1.0p-48, offset);
    }
  }
}

cudaError_t launch_rand_block(const long long *seeds, int npart, long long rows, int cols, double offset,
                              double *A, long long lda, cudaStream_t s) {
  const long long total = (long long)npart * rows;
  if (total == 0 || cols == 0) return cudaSuccess;
  const int grid = (int)std::min<long long>(ceil_div(total, 256), 152 * 16);
  HODLR_LAUNCH(rand_block_kernel, grid, 256, 0, s, seeds, npart, rows, cols, offset, A, lda);
  return cudaGetLastError();
}

// DenseBlockTask (src/tasks/dense_block.cc:63-75) with the reference's BLAS
// loop order (netlib DGEMM 'N','T' with beta = 0: for each column j, the
// products U(i,l) V(j,l) added into a zeroed column in the order l = 0 ..
// r-1), then the diagonal D added: K_leaf = U_leaf V_leaf^T + diag(D_leaf).
// Separate rounded multiplies and adds (no fused multiply-add), so the
// blocks equal the reference's bit for bit.
__global__ void seeded_leaves_kernel(const double *__restrict__ U, const double *__restrict__ V,
                                     const double *__restrict__ Dg, long long n, int m, int r, int nleaf,
                                     double *K) {
  const long long mm = (long long)m * m, total = (long long)nleaf * mm;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long k = e / mm, w = e % mm;
    const int i = (int)(w % m), j = (int)(w / m);
    const double *u = U + k * m + i, *v = V + k * m + j;
    double c = 0.0;
    for (int l = 0; l < r; ++l) c = __dadd_rn(c, __dmul_rn(v[(long long)l * n], u[(long long)l * n]));
    if (i == j) c = __dadd_rn(c, Dg[k * m + i]);
    K[e] = c;
  }
}

cudaError_t launch_seeded_leaves(const double *U, const double *V, const double *Dg, long long n, int m, int r,
                                 int nleaf, double *K, cudaStream_t s) {
  const long long total = (long long)nleaf * m * m;
  if (total == 0) return cudaSuccess;
  const int grid = (int)std::min<long long>(ceil_div(total, 256), 152 * 16);
  HODLR_LAUNCH(seeded_leaves_kernel, grid, 256, 0, s, U, V, Dg, n, m, r, nleaf, K);
  return cudaGetLastError();
}

}  // namespace hodlr
