// C++ driver of the irregular tree (hodlr_gb300::IrregularTree): the matrix
// of fastSolver2's SPMD drivers with one heavy shard and unequal shard ranks
// (spmd_driver/solver_irregular_part.cc, solver_irregular_ranks.cc) -- two
// shards, shard 0 with leaf 32 and rank 4, shard 1 with ten times the leaf
// and rank 6, coupled with ranks (5, 3) -- set from host buffers, factored
// and solved in FP64; prints one JSON line with ||b - A x|| / ||b|| from the
// tree's own FP64 product and the LMatrix-style unequal-rank node solve
// checked against its definition on one node.
//   usage: test_tree
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "hodlr_gb300.hpp"

using hodlr_gb300::IrregularTree;

namespace {

struct Rng {  // xorshift64*: seeded uniform values in [-1, 1)
  unsigned long long s;
  double next() {
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    return (double)((s * 2685821657736338717ULL) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
};

double *to_device(const std::vector<double> &h) {
  double *d = nullptr;
  cudaMalloc(&d, sizeof(double) * h.size());
  cudaMemcpy(d, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice);
  return d;
}

std::vector<double> random_matrix(Rng &g, long long rows, int cols, double scale) {
  std::vector<double> a((size_t)rows * cols);
  for (auto &x : a) x = scale * g.next();
  return a;
}

}  // namespace

int main() {
  Rng g{0x9e3779b97f4a7c15ULL};
  const int levels = 3, nrhs = 4;
  const int leaf[2] = {32, 320}, rank[2] = {4, 6};
  std::vector<hodlr_desc> shards(2);
  for (int j = 0; j < 2; ++j) {
    shards[j] = hodlr_desc{};
    shards[j].n = (int64_t)leaf[j] << levels;
    shards[j].leaf = leaf[j];
    shards[j].levels = levels;
    shards[j].rank = rank[j];
    shards[j].precision = HODLR_PREC_FP64;
  }
  const std::vector<int32_t> coupling = {5, 3};
  IrregularTree tree(1, shards, coupling, nrhs);
  std::vector<double *> keep;
  for (int j = 0; j < 2; ++j) {
    const int m = leaf[j];
    const long long n = shards[j].n;
    std::vector<double> K((size_t)n * m);  // KTree layout: leaf i at rows i*m, ld n
    for (long long i = 0; i < n; ++i)
      for (int c = 0; c < m; ++c) K[i + (long long)c * n] = g.next() / std::sqrt((double)m) + (i % m == c ? 4.0 : 0.0);
    keep.push_back(to_device(K));
    tree.set_leaf_blocks(j, keep.back(), n, m);
    for (int l = 0; l < levels; ++l) {
      const double sc = 1.0 / std::sqrt((double)(n >> (l + 1)));
      keep.push_back(to_device(random_matrix(g, n, rank[j], sc)));
      double *U = keep.back();
      keep.push_back(to_device(random_matrix(g, n, rank[j], sc)));
      tree.set_level(j, l, U, n, keep.back(), n);
    }
  }
  for (int h = 0; h < 2; ++h) {  // U_c with its own rank, V_c with the sibling's
    const long long n = shards[h].n;
    const double sc = 1.0 / std::sqrt((double)n);
    keep.push_back(to_device(random_matrix(g, n, coupling[h], sc)));
    double *U = keep.back();
    keep.push_back(to_device(random_matrix(g, n, coupling[1 - h], sc)));
    tree.set_coupling(0, 0, h, U, n, keep.back(), n);
  }
  const long long N = tree.rows();
  std::vector<double> b = random_matrix(g, N, nrhs, 1.0);
  double *X = to_device(b), *Y = nullptr;
  cudaMalloc(&Y, sizeof(double) * N * nrhs);
  tree.factor();
  tree.solve(X, N, nrhs);
  tree.matvec(X, N, Y, N, nrhs);
  std::vector<double> y((size_t)N * nrhs);
  cudaMemcpy(y.data(), Y, sizeof(double) * y.size(), cudaMemcpyDeviceToHost);
  double rmax = 0.0;
  for (int c = 0; c < nrhs; ++c) {
    double rn = 0.0, bn = 0.0;
    for (long long i = 0; i < N; ++i) {
      const double d = b[i + c * N] - y[i + c * N];
      rn += d * d;
      bn += b[i + c * N] * b[i + c * N];
    }
    rmax = std::fmax(rmax, std::sqrt(rn / bn));
  }
  // one unequal-rank node solve against its definition: S [eta0; eta1] = [VTd1; VTd0]
  const int r0 = 3, r1 = 2;
  std::vector<double> u0 = random_matrix(g, r1, r0, 0.3), u1 = random_matrix(g, r0, r1, 0.3);
  std::vector<double> d0 = random_matrix(g, r1, 1, 1.0), d1 = random_matrix(g, r0, 1, 1.0);
  double *du0 = to_device(u0), *du1 = to_device(u1), *dd0 = to_device(d0), *dd1 = to_device(d1);
  hodlr_gb300::LMatrix::node_solve(1, r0, r1, 1, du0, r1, du1, r0, dd0, r1, dd1, r0);
  std::vector<double> e0(r1), e1(r0);
  cudaMemcpy(e0.data(), dd0, sizeof(double) * r1, cudaMemcpyDeviceToHost);
  cudaMemcpy(e1.data(), dd1, sizeof(double) * r0, cudaMemcpyDeviceToHost);
  double node_err = 0.0;  // rows of S: [I, VTu1] eta = VTd1 and [VTu0, I] eta = VTd0, eta = [e1; e0]
  for (int i = 0; i < r0; ++i) {
    double s = e1[i];
    for (int j = 0; j < r1; ++j) s += u1[i + j * r0] * e0[j];
    node_err = std::fmax(node_err, std::fabs(s - d1[i]));
  }
  for (int j = 0; j < r1; ++j) {
    double s = e0[j];
    for (int i = 0; i < r0; ++i) s += u0[j + i * r1] * e1[i];
    node_err = std::fmax(node_err, std::fabs(s - d0[j]));
  }
  std::printf("{\"rows\": %lld, \"rel_residual\": %.3e, \"node_solve_err\": %.3e}\n", N, rmax, node_err);
  for (double *p : keep) cudaFree(p);
  for (double *p : {X, Y, du0, du1, dd0, dd1}) cudaFree(p);
  return 0;
}
