// Element-wise and bookkeeping kernels of the sweeps: precision
// conversions, leaf packing, copies / corrections, deterministic column
// norms and the device-side refinement control, the input scan for
// non-finite values, and the scale-gradient reduction of the adjoint.
#include <algorithm>

#include "dense_ops.cuh"
#include "kernels.cuh"

namespace hodlr {

// --------------------------------------------------------------- helpers
template <typename Tout, typename Tin> __device__ __forceinline__ Tout convert_one(Tin x) { return (Tout)x; }
template <> __device__ __forceinline__ float convert_one<float, double>(double x) { return f64_to_f32_rn(x); }

template <typename Tin, typename Tout>
__global__ void convert_kernel(const Tin *X, long long ldx, Tout *Y, long long ldy, long long n, int c) {
  HODLR_FOR_2D(i, j, n, c) Y[i + j * ldy] = convert_one<Tout>(X[i + j * ldx]);
}

static int grid_for(long long total) {
  return (int)std::max<long long>(1, std::min<long long>(ceil_div(total, 256), 152 * 16));
}

template <typename Tin, typename Tout>
cudaError_t launch_convert(const Tin *X, long long ldx, Tout *Y, long long ldy, long long n, int c,
                           cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH((convert_kernel<Tin, Tout>), grid2d(n, c), 256, 0, s, X, ldx, Y, ldy, n, c);
  return cudaGetLastError();
}
template cudaError_t launch_convert<double, float>(const double *, long long, float *, long long, long long,
                                                   int, cudaStream_t);
template cudaError_t launch_convert<float, double>(const float *, long long, double *, long long, long long,
                                                   int, cudaStream_t);
template cudaError_t launch_convert<double, double>(const double *, long long, double *, long long,
                                                    long long, int, cudaStream_t);

__global__ void pack_leaves_kernel(const double *D, long long ld, long long stride, double *out, int m,
                                   long long total) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long mm = (long long)m * m;
    const long long leaf = e / mm, w = e % mm;
    const int i = (int)(w % m), j = (int)(w / m);
    out[e] = D[leaf * stride + i + (long long)j * ld];
  }
}

cudaError_t launch_pack_leaves(const double *D, long long ld, long long stride, double *out, int m,
                               int nleaf, cudaStream_t s) {
  const long long total = (long long)nleaf * m * m;
  HODLR_LAUNCH(pack_leaves_kernel, grid_for(total), 256, 0, s, D, ld, stride, out, m, total);
  return cudaGetLastError();
}

template <typename T>
__global__ void unpack_leaves_kernel(const T *in, double *out, long long ld, long long stride, int m,
                                     long long total) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long mm = (long long)m * m;
    const long long leaf = e / mm, w = e % mm;
    const int i = (int)(w % m), j = (int)(w / m);
    out[leaf * stride + i + (long long)j * ld] = (double)in[e];
  }
}

template <typename T>
cudaError_t launch_unpack_leaves(const T *in, double *out, long long ld, long long stride, int m, int nleaf,
                                 cudaStream_t s) {
  const long long total = (long long)nleaf * m * m;
  HODLR_LAUNCH(unpack_leaves_kernel<T>, grid_for(total), 256, 0, s, in, out, ld, stride, m, total);
  return cudaGetLastError();
}
template cudaError_t launch_unpack_leaves<double>(const double *, double *, long long, long long, int, int,
                                                  cudaStream_t);
template cudaError_t launch_unpack_leaves<float>(const float *, double *, long long, long long, int, int,
                                                 cudaStream_t);

__global__ void axpy_kernel(const double *X, long long ldx, double *Y, long long ldy, long long n, int c,
                            double alpha, int accumulate, const int *skip) {
  if (skip && *skip) return;
  HODLR_FOR_2D(i, j, n, c) {
    const double v = X[i + j * ldx];
    double *y = Y + i + j * ldy;
    *y = accumulate ? *y + alpha * v : alpha * v;
  }
}

cudaError_t launch_axpy(const double *X, long long ldx, double *Y, long long ldy, long long n, int c,
                        double alpha, bool accumulate, const int *skip, cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH(axpy_kernel, grid2d(n, c), 256, 0, s, X, ldx, Y, ldy, n, c, alpha, (int)accumulate, skip);
  return cudaGetLastError();
}

template <typename Td>
__global__ void add_corr_kernel(const double *X, long long ldx, const Td *D, long long ldd, double *Y,
                                long long ldy, long long n, int c, const int *skip) {
  if (skip && *skip) return;
  HODLR_FOR_2D(i, j, n, c) Y[i + j * ldy] = X[i + j * ldx] + (double)D[i + j * ldd];
}

template <typename Td>
cudaError_t launch_add_correction(const double *X, long long ldx, const Td *D, long long ldd, double *Y,
                                  long long ldy, long long n, int c, const int *skip, cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH(add_corr_kernel<Td>, grid2d(n, c), 256, 0, s, X, ldx, D, ldd, Y, ldy, n, c, skip);
  return cudaGetLastError();
}
template cudaError_t launch_add_correction<float>(const double *, long long, const float *, long long, double *,
                                                  long long, long long, int, const int *, cudaStream_t);
template cudaError_t launch_add_correction<double>(const double *, long long, const double *, long long,
                                                   double *, long long, long long, int, const int *,
                                                   cudaStream_t);

// Column sums of squares in two deterministic passes: per (column, slice)
// partial sums, then a fixed-order sum per column.
static constexpr int kNormSlices = 64;

__global__ void colnorm_partial_kernel(const double *X, long long ldx, long long n, double *work,
                                       const int *skip) {
  if (skip && *skip) return;
  const int j = blockIdx.y, sl = blockIdx.x;
  const long long per = (n + kNormSlices - 1) / kNormSlices;
  const long long lo = sl * per, hi = min(n, lo + per);
  double acc = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double v = X[i + (long long)j * ldx];
    acc += v * v;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) work[(long long)j * kNormSlices + sl] = red[0];
}

__global__ void colnorm_final_kernel(const double *work, int c, double *out, const int *skip) {
  if (skip && *skip) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= c) return;
  double s = 0.0;
  for (int k = 0; k < kNormSlices; ++k) s += work[(long long)j * kNormSlices + k];
  out[j] = sqrt(s);
}

cudaError_t launch_colnorms(const double *X, long long ldx, long long n, int c, double *out, double *work,
                            const int *skip, cudaStream_t s) {
  if (c <= 0) return cudaSuccess;
  HODLR_LAUNCH(colnorm_partial_kernel, dim3(kNormSlices, c), 256, 0, s, X, ldx, n, work, skip);
  HODLR_LAUNCH(colnorm_final_kernel, ceil_div(c, 64), 64, 0, s, work, c, out, skip);
  return cudaGetLastError();
}

// One warp per (leaf, column): the sum of squares of the leaf's m rows, in a
// fixed butterfly order.
__global__ void leaf_sumsq_kernel(const double *X, long long ldx, int m, int nleaf, int c, double *work,
                                  const int *skip) {
  if (skip && *skip) return;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= (long long)nleaf * c) return;
  const int leaf = (int)(w % nleaf), j = (int)(w / nleaf);
  const double *x = X + (long long)leaf * m + (long long)j * ldx;
  double acc = 0.0;
  for (int i = lane; i < m; i += 32) acc += x[i] * x[i];
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) work[(long long)j * nleaf + leaf] = acc;
}

__global__ void seg_norm_kernel(const double *work, int nleaf, int c, const int *seg, int nsys, double *out,
                                const int *skip) {
  if (skip && *skip) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nsys * c) return;
  const int i = t % nsys, j = t / nsys;
  double acc = 0.0;
  for (int q = seg[i]; q < seg[i + 1]; ++q) acc += work[(long long)j * nleaf + q];
  out[(long long)j * nsys + i] = sqrt(acc);
}

cudaError_t launch_seg_colnorms(const double *X, long long ldx, int m, int nleaf, int c, const int *seg_leaf,
                                int nsys, double *out, double *work, const int *skip, cudaStream_t s) {
  if (c <= 0 || nleaf <= 0) return cudaSuccess;
  const long long warps = (long long)nleaf * c;
  HODLR_LAUNCH(leaf_sumsq_kernel, (int)ceil_div(warps * 32, 256), 256, 0, s, X, ldx, m, nleaf, c, work, skip);
  HODLR_LAUNCH(seg_norm_kernel, ceil_div(nsys * c, 128), 128, 0, s, work, nleaf, c, seg_leaf, nsys, out, skip);
  return cudaGetLastError();
}

__global__ void scale_cols_kernel(double *X, long long ldx, long long n, int c, const double *sc) {
  HODLR_FOR_2D(i, j, n, c) X[i + j * ldx] *= sc[j];
}

cudaError_t launch_scale_cols(double *X, long long ldx, long long n, int c, const double *sc, cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH(scale_cols_kernel, grid2d(n, c), 256, 0, s, X, ldx, n, c, sc);
  return cudaGetLastError();
}

// grid (row chunks, systems): each CTA strides over its system's n x kmax
// elements (one column-major sweep per column).
__global__ void gather_rhs_kernel(const RhsCopy *tab, double *G, long long ldg, int kmax) {
  const RhsCopy t = tab[blockIdx.y];
  const long long total = t.n * kmax;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e % t.n;
    const int j = (int)(e / t.n);
    G[t.row_off + i + j * ldg] = j < t.k ? t.ext[i + j * t.ld] : 0.0;
  }
}

__global__ void scatter_rhs_kernel(const RhsCopy *tab, const double *G, long long ldg) {
  const RhsCopy t = tab[blockIdx.y];
  const long long total = t.n * t.k;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e % t.n;
    const int j = (int)(e / t.n);
    t.ext[i + j * t.ld] = G[t.row_off + i + j * ldg];
  }
}

static dim3 rhs_grid(int count, long long maxn, int kmax) {
  const long long chunks = std::max<long long>(1, std::min<long long>(ceil_div(maxn * kmax, 256), 64));
  return dim3((unsigned)chunks, (unsigned)count);
}

cudaError_t launch_gather_rhs(const RhsCopy *tab, int count, long long maxn, double *G, long long ldg, int kmax,
                              cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  HODLR_LAUNCH(gather_rhs_kernel, rhs_grid(count, maxn, kmax), 256, 0, s, tab, G, ldg, kmax);
  return cudaGetLastError();
}

cudaError_t launch_scatter_rhs(const RhsCopy *tab, int count, long long maxn, const double *G, long long ldg,
                               int kmax, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  HODLR_LAUNCH(scatter_rhs_kernel, rhs_grid(count, maxn, kmax), 256, 0, s, tab, G, ldg);
  return cudaGetLastError();
}

// Fused passes of the refinement loop.  Partial sums of squares per (row
// block, column): P blocks of `per` rows (64 slices for one system, one leaf
// per block for a forest), each summed by its CTA in a fixed order.
__device__ __forceinline__ void block_sumsq_store(double acc, double *work, long long idx) {
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) work[idx] = red[0];
}

// B64 = B, X32 = fl32(B), partial sums of squares of B
__global__ void rhs_prepare_kernel(const double *B, long long ldb, long long n, int P, long long per,
                                   double *B64, float *X32, double *work) {
  const int j = blockIdx.y, pb = blockIdx.x;
  const long long lo = pb * per, hi = min(n, lo + per);
  double acc = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double v = B[i + (long long)j * ldb];
    B64[i + (long long)j * n] = v;
    X32[i + (long long)j * n] = f64_to_f32_rn(v);
    acc += v * v;
  }
  block_sumsq_store(acc, work, (long long)j * P + pb);
}

cudaError_t launch_rhs_prepare(const double *B, long long ldb, long long n, int k, int P, double *B64, float *X32,
                               double *work, cudaStream_t s) {
  if (n <= 0 || k <= 0) return cudaSuccess;
  const long long per = (n + P - 1) / P;
  HODLR_LAUNCH(rhs_prepare_kernel, dim3(P, k), 256, 0, s, B, ldb, n, P, per, B64, X32, work);
  return cudaGetLastError();
}

// R = hi + lo of the double-word residual: X32 = fl32(R) (the correction's
// right-hand side) and the partial sums of squares of R
__global__ void resid_finish_kernel(const float2 *R2, long long n, int P, long long per, float *X32, double *work,
                                    const int *skip) {
  if (skip && *skip) return;
  const int j = blockIdx.y, pb = blockIdx.x;
  const long long lo = pb * per, hi = min(n, lo + per);
  // FP32 arithmetic only (GB300's FP64 pipe runs at 1/64 of the FP32 rate):
  // hi + lo rounds the normalised double-word value to FP32 correctly; the
  // squares accumulate per thread in FP32 relative to a running power-of-two
  // scale sc > max |v| (the scale / sum-of-squares scheme of nrm2, every
  // rescaling exact), so residuals of any magnitude neither underflow nor
  // overflow; the block combines ssq sc^2 in FP64
  float sc = 0.f, isc = 0.f, ssq = 0.f;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const float2 rv = R2[i + (long long)j * n];
    const float v = rv.x + rv.y;
    X32[i + (long long)j * n] = v;
    const float av = fabsf(v);
    if (av >= sc && av > 0.f && av <= 3.4028235e38f) {
      const int eb = (int)((__float_as_uint(av) >> 23) & 0xff);  // sc = 2^(e + 1) > |v|, at most 2^127
      const int es = eb < 254 ? eb + 1 : 254;
      const float ns = __uint_as_float((unsigned)es << 23), ins = __uint_as_float((unsigned)(254 - es) << 23);
      const float rr = sc * ins;  // old / new scale (a power of two <= 1)
      ssq *= rr * rr;
      sc = ns;
      isc = ins;
    }
    const float t = v * isc;
    ssq = fmaf(t, t, ssq);
  }
  block_sumsq_store((double)ssq * (double)sc * (double)sc, work, (long long)j * P + pb);
}

cudaError_t launch_resid_finish(const float2 *R2, long long n, int k, int P, float *X32, double *work,
                                const int *skip, cudaStream_t s) {
  if (n <= 0 || k <= 0) return cudaSuccess;
  const long long per = (n + P - 1) / P;
  HODLR_LAUNCH(resid_finish_kernel, dim3(P, k), 256, 0, s, R2, n, P, per, X32, work, skip);
  return cudaGetLastError();
}

// out[j*nseg + i] = sqrt(sum of the partials of segment i of column j); one
// segment covering all P partials gives plain column norms
cudaError_t launch_partial_norms(const double *work, int P, int k, const int *seg, int nseg, double *out,
                                 const int *skip, cudaStream_t s);

__global__ void refine_check_kernel(const double *rnorm, const double *bnorm, int c, double tol,
                                    DevStatus *st, int advance) {
  if (threadIdx.x != 0) return;
  if (st->done) return;
  double rel = 0.0;
  for (int j = 0; j < c; ++j) {
    const double b = bnorm[j] > 0.0 ? bnorm[j] : 1.0;
    const double q = rnorm[j] / b;
    rel = (q > rel || q != q) ? q : rel;
  }
  st->resid = rel;
  if (rel <= tol) st->done = 1;
  if (advance && !st->done) st->iters += 1;
}

__global__ void partial_norm_final_kernel(const double *work, int P, int k, double *out, const int *skip) {
  if (skip && *skip) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  double acc = 0.0;
  for (int q = 0; q < P; ++q) acc += work[(long long)j * P + q];
  out[j] = sqrt(acc);
}

cudaError_t launch_partial_norms(const double *work, int P, int k, const int *seg, int nseg, double *out,
                                 const int *skip, cudaStream_t s) {
  if (k <= 0) return cudaSuccess;
  if (!seg) {
    HODLR_LAUNCH(partial_norm_final_kernel, ceil_div(k, 64), 64, 0, s, work, P, k, out, skip);
  } else {
    HODLR_LAUNCH(seg_norm_kernel, ceil_div(nseg * k, 128), 128, 0, s, work, P, k, seg, nseg, out, skip);
  }
  return cudaGetLastError();
}

cudaError_t launch_refine_check(const double *rnorm, const double *bnorm, int c, double tol, DevStatus *st,
                                int advance, cudaStream_t s) {
  HODLR_LAUNCH(refine_check_kernel, 1, 32, 0, s, rnorm, bnorm, c, tol, st, advance);
  return cudaGetLastError();
}

__global__ void refine_check_cond_kernel(const double *rnorm, const double *bnorm, int c, double tol,
                                         DevStatus *st, int maxit, cudaGraphConditionalHandle cond) {
  if (threadIdx.x != 0) return;
  unsigned more = 0;
  if (!st->done) {
    double rel = 0.0;
    for (int j = 0; j < c; ++j) {
      const double b = bnorm[j] > 0.0 ? bnorm[j] : 1.0;
      const double q = rnorm[j] / b;
      rel = (q > rel || q != q) ? q : rel;
    }
    st->resid = rel;
    if (rel <= tol) {
      st->done = 1;
    } else if (st->iters < maxit) {
      st->iters += 1;
      more = 1;
    }
  }
  cudaGraphSetConditional(cond, more);
}

cudaError_t launch_refine_check_cond(const double *rnorm, const double *bnorm, int c, double tol, DevStatus *st,
                                     int maxit, cudaGraphConditionalHandle cond, cudaStream_t s) {
  HODLR_LAUNCH(refine_check_cond_kernel, 1, 32, 0, s, rnorm, bnorm, c, tol, st, maxit, cond);
  return cudaGetLastError();
}

__global__ void check_finite_kernel(const double *X, long long ldx, long long n, int c, DevStatus *st) {
  HODLR_FOR_2D(i, j, n, c) {
    if (!isfinite(X[i + j * ldx])) report_error(st, HODLR_ERR_NONFINITE_INPUT, i);
  }
}

cudaError_t launch_check_finite(const double *X, long long ldx, long long n, int c, DevStatus *st,
                                cudaStream_t s) {
  if (n * c == 0) return cudaSuccess;
  HODLR_LAUNCH(check_finite_kernel, grid2d(n, c), 256, 0, s, X, ldx, n, c, st);
  return cudaGetLastError();
}

__global__ void fill_kernel(double *X, long long n, double v) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    X[e] = v;
}

__global__ void add_leaf_diag_kernel(double *D, const double *d, int m, long long total) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long leaf = e / m;
    const int j = (int)(e - leaf * m);
    D[leaf * m * m + (long long)j * (m + 1)] += d[e];
  }
}

cudaError_t launch_add_leaf_diag(double *D, const double *d, int m, int nleaf, cudaStream_t s) {
  const long long total = (long long)nleaf * m;
  HODLR_LAUNCH(add_leaf_diag_kernel, grid_for(total), 256, 0, s, D, d, m, total);
  return cudaGetLastError();
}

cudaError_t launch_fill(double *X, long long n, double v, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  HODLR_LAUNCH(fill_kernel, grid_for(n), 256, 0, s, X, n, v);
  return cudaGetLastError();
}

// One CTA per rank index j; the batches are strided over the threads and the
// partial sums combined in a fixed-order tree (deterministic).
__global__ void scale_grad_kernel(const double *W, const double *T, int r, int k, int nbatch, double *ds) {
  const int j = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nbatch; b += blockDim.x) {
    const double *w = W + (long long)b * r * k;
    const double *t = T + (long long)(b ^ 1) * r * k;
    for (int q = 0; q < k; ++q) acc += w[j + (long long)q * r] * t[j + (long long)q * r];
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) ds[j] = -red[0];
}

cudaError_t launch_scale_grad(const double *W, const double *T, int r, int k, int nbatch, double *ds,
                              cudaStream_t s) {
  HODLR_LAUNCH(scale_grad_kernel, r, 256, 0, s, W, T, r, k, nbatch, ds);
  return cudaGetLastError();
}

// ------------------------------------------------- unequal leaf sizes
// Rows of leaf i (rows off[i] .. off[i] + sz[i] of a packed matrix) to or
// from rows i * mp .. of the padded one; padded rows are zero.
__global__ void pad_rows_kernel(const long long *off, const int *sz, int nleaf, int mp, int cols, const double *src,
                                long long lds, double *dst, long long ldd, int unpad) {
  const long long total = (long long)nleaf * mp;
  for (long long j = blockIdx.y; j < cols; j += gridDim.y)
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
      const int i = (int)(e / mp), q = (int)(e % mp);
      const bool real = q < sz[i];
      const long long pr = e, rr = off[i] + q;  // padded row, packed row
      if (!unpad)
        dst[pr + j * ldd] = real ? src[rr + j * lds] : 0.0;
      else if (real)
        dst[rr + j * ldd] = src[pr + j * lds];
    }
}

cudaError_t launch_pad_rows(const long long *off, const int *sz, int nleaf, int mp, int cols, const double *src,
                            long long lds, double *dst, long long ldd, bool unpad, cudaStream_t s) {
  const long long total = (long long)nleaf * mp;
  if (total == 0 || cols == 0) return cudaSuccess;
  dim3 grid((unsigned)std::min<long long>(ceil_div(total, 256), 152 * 8), (unsigned)std::min(cols, 65535));
  HODLR_LAUNCH(pad_rows_kernel, grid, 256, 0, s, off, sz, nleaf, mp, cols, src, lds, dst, ldd, unpad ? 1 : 0);
  return cudaGetLastError();
}

// Leaf blocks packed one after another (block i: sz[i] x sz[i], column-major,
// starting at boff[i]) into [nleaf][mp][mp] with an identity on the padding.
__global__ void pad_leaf_blocks_kernel(const long long *boff, const int *sz, int nleaf, int mp, const double *src,
                                       double *dst) {
  const long long mm = (long long)mp * mp, total = (long long)nleaf * mm;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / mm);
    const int w = (int)(e % mm), r = w % mp, c = w / mp, m = sz[i];
    dst[e] = (r < m && c < m) ? src[boff[i] + r + (long long)c * m] : (r == c ? 1.0 : 0.0);
  }
}

cudaError_t launch_pad_leaf_blocks(const long long *boff, const int *sz, int nleaf, int mp, const double *src,
                                   double *dst, cudaStream_t s) {
  const long long total = (long long)nleaf * mp * mp;
  if (total == 0) return cudaSuccess;
  HODLR_LAUNCH(pad_leaf_blocks_kernel, (unsigned)std::min<long long>(ceil_div(total, 256), 152 * 16), 256, 0, s,
               boff, sz, nleaf, mp, src, dst);
  return cudaGetLastError();
}

}  // namespace hodlr
