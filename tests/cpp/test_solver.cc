// C++ driver mirroring fastSolver2's test_solver (tests/test.cc:544-661) on
// the GB300 library: reference-structured inputs from drand48 streams (one
// seed per leaf partition, D + 1e3, one U and V for all levels), then
// HMatrix(nProc, level).init(U, V, D) and solve(b), and the residual
// ||b - (U (V^T x) + D.x)|| / ||b|| that the reference leaves disabled
// (tests/test.cc:651-658); then the same problem built on the device from
// its seeds (HMatrix::init_seeded) and a checkpoint round trip of that
// factorisation.  Prints one JSON line; with a fourth argument it writes x
// (raw float64) to that file.
//   usage: test_solver <leaf> <levels> <rank> [x.bin]
#include <cuda_runtime.h>
#include <stdlib.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "hodlr_gb300.hpp"

static std::vector<long> seeds(long master, int n) {
  drand48_data buf;
  srand48_r(master, &buf);
  std::vector<long> s(n);
  for (auto &x : s) lrand48_r(&buf, &x);
  return s;
}

// Matrix(base, level, cols).rand(): block k (base rows) from seeds[k], filled
// row by row (src/ptr_matrix.cc:62-71).
static std::vector<double> rand_matrix(const std::vector<long> &sd, int base, int cols, int offset) {
  const long long n = (long long)sd.size() * base;
  std::vector<double> A(n * cols);
  for (size_t k = 0; k < sd.size(); ++k) {
    drand48_data buf;
    srand48_r(sd[k], &buf);
    for (int i = 0; i < base; ++i)
      for (int j = 0; j < cols; ++j) {
        double v;
        drand48_r(&buf, &v);
        A[(long long)k * base + i + (long long)j * n] = v + offset;
      }
  }
  return A;
}

int main(int argc, char **argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s leaf levels rank [x.bin]\n", argv[0]);
    return 2;
  }
  const int leaf = atoi(argv[1]), level = atoi(argv[2]), rank = atoi(argv[3]);
  const int nPart = 1 << level;
  const long long N = (long long)leaf * nPart;
  const long master = 20240601;
  auto V = rand_matrix(seeds(master + 0, nPart), leaf, rank, 0);
  auto U = rand_matrix(seeds(master + 1, nPart), leaf, rank, 0);
  auto b = rand_matrix(seeds(master + 2, nPart), leaf, 1, 0);
  auto D = rand_matrix(seeds(master + 3, nPart), leaf, 1, 1000);
  try {
    hodlr_gb300::HMatrix H(/*nProc=*/std::min(nPart, 8), level);
    H.init(U.data(), V.data(), D.data(), N, rank);
    double *dB = nullptr, *dY = nullptr;
    if (cudaMalloc(&dB, sizeof(double) * N) != cudaSuccess || cudaMalloc(&dY, sizeof(double) * N) != cudaSuccess)
      throw hodlr_gb300::Error(HODLR_ERR_OUT_OF_MEMORY, "cudaMalloc");
    cudaMemcpy(dB, b.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
    H.solve(dB, N, 1);
    H.matvec(dB, N, dY, N, 1);
    std::vector<double> x(N), y(N);
    cudaMemcpy(x.data(), dB, sizeof(double) * N, cudaMemcpyDeviceToHost);
    cudaMemcpy(y.data(), dY, sizeof(double) * N, cudaMemcpyDeviceToHost);
    double rn = 0, bn = 0, xs = 0;
    for (long long i = 0; i < N; ++i) {
      rn += (b[i] - y[i]) * (b[i] - y[i]);
      bn += b[i] * b[i];
      xs += x[i];
    }
    // the same problem from its seeds on the device (HMatrix::init_seeded),
    // then a checkpoint of that factorisation restored into a third HMatrix
    auto to64 = [](const std::vector<long> &v) { return std::vector<int64_t>(v.begin(), v.end()); };
    const auto vs = to64(seeds(master + 0, nPart)), us = to64(seeds(master + 1, nPart)),
               ds = to64(seeds(master + 3, nPart));
    hodlr_gb300::HMatrix H2(/*nProc=*/1, level), H3(/*nProc=*/1, level);
    H2.init_seeded(us.data(), vs.data(), ds.data(), N, rank, 1000.0);
    std::vector<double> x2(N), x3(N);
    cudaMemcpy(dB, b.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
    H2.solve(dB, N, 1);
    cudaMemcpy(x2.data(), dB, sizeof(double) * N, cudaMemcpyDeviceToHost);
    H3.restore(H2.checkpoint());
    cudaMemcpy(dB, b.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
    H3.solve(dB, N, 1);
    cudaMemcpy(x3.data(), dB, sizeof(double) * N, cudaMemcpyDeviceToHost);
    double dn = 0, xn = 0;
    bool same = true;
    for (long long i = 0; i < N; ++i) {
      dn += (x2[i] - x[i]) * (x2[i] - x[i]);
      xn += x[i] * x[i];
      same = same && x3[i] == x2[i];
    }
    printf("{\"n\": %lld, \"leaf\": %d, \"levels\": %d, \"rank\": %d, \"rel_residual\": %.6e, \"x_sum\": %.17g, "
           "\"seeded_rel_diff\": %.6e, \"checkpoint_identical\": %s}\n",
           N, leaf, level, rank, std::sqrt(rn / bn), xs, std::sqrt(dn / xn), same ? "true" : "false");
    if (argc > 4) {
      FILE *f = fopen(argv[4], "wb");
      if (!f || fwrite(x.data(), sizeof(double), N, f) != (size_t)N) return 3;
      fclose(f);
    }
    cudaFree(dB);
    cudaFree(dY);
  } catch (const hodlr_gb300::Error &e) {
    fprintf(stderr, "error %d: %s\n", e.code, e.what());
    return 1;
  }
  return 0;
}
