// hodlr_gb300.hpp -- C++ host library over the C ABI (header only).
//
// Keeps fastSolver2's host-side vocabulary so its drivers port line by line:
//   HMatrix(nProc, level); init(U, V, D); solve(b)     include/hmatrix.hpp:10-23
//   LMatrix::gemmRed / gemmBro / node_solve             include/lmatrix.hpp:119-169
//   KTree::solve (leaf solve), hsolve                   include/tree.hpp:362-389,
//                                                       src/tasks/leaf_solve.cc:8-10
//   the SPMD drivers' per-shard subtrees under top levels with unequal
//   sibling ranks (IrregularTree)                       spmd_driver/solver_irregular_part.cc,
//                                                       spmd_driver/solver_irregular_ranks.cc
// The Legion context/runtime arguments are gone (one process, one GPU); the
// matrices are plain column-major buffers (host or device), and failures
// throw hodlr_gb300::Error instead of asserting.
#ifndef HODLR_GB300_HPP
#define HODLR_GB300_HPP

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "hodlr_gb300.h"

namespace hodlr_gb300 {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int status) {
  if (status != HODLR_OK) throw Error(status, hodlr_last_error_string());
}

// The reference's raw-pointer solve, in place (see hodlr_hsolve).
inline void hsolve(int nrow, int nrhs, int rank, int nPart, int LD, double *K, double *U, double *V) {
  check(hodlr_hsolve(nrow, nrhs, rank, nPart, LD, K, U, V));
}

// A = blockdiag(D_leaf) + hierarchical off-diagonal low rank, factored once
// and solved many times.
class HMatrix {
 public:
  HMatrix() = default;
  // nProc is the reference's processor count (it must divide 2^level there,
  // src/hmatrix.cc:16-19); one GPU solves the whole tree here, it is checked
  // and otherwise unused.
  HMatrix(int nProc, int level) : level_(level) {
    if (nProc < 1 || ((1 << level) % nProc) != 0) throw Error(HODLR_ERR_INVALID_ARG, "nProc must divide 2^level");
  }
  HMatrix(const HMatrix &) = delete;
  HMatrix &operator=(const HMatrix &) = delete;
  ~HMatrix() { destroy(); }

  // The reference's HMatrix::init(U, V, D): A = U V^T + diag(D) with
  // N = U's rows, leaf = N / 2^level (src/hmatrix.cc:22-47).
  void init(const double *U, const double *V, const double *D, int64_t N, int rank, int nrhs_max = 1,
            int precision = HODLR_PREC_FP64) {
    create(N, rank, nrhs_max, precision);
    check(hodlr_set_uvd(h_, U, N, V, N, D));
    factored_ = false;
  }

  // HMatrix::init from the per-leaf seeds of the reference's MapSeed
  // argument maps (src/lmatrix.cc:327-360): U, V, D and the leaf blocks
  // built on the device bit for bit as the reference's tasks build them.
  void init_seeded(const int64_t *useeds, const int64_t *vseeds, const int64_t *dseeds, int64_t N, int rank,
                   double offset, int nrhs_max = 1, int precision = HODLR_PREC_FP64) {
    create(N, rank, nrhs_max, precision);
    check(hodlr_set_seeded(h_, useeds, vseeds, dseeds, offset));
    factored_ = false;
  }

  // The factored state as bytes, and a factored HMatrix from them.
  std::vector<char> checkpoint() {
    if (!factored_) factor();
    int64_t nb = 0;
    check(hodlr_checkpoint_size(h_, &nb));
    std::vector<char> buf((size_t)nb);
    check(hodlr_checkpoint_save(h_, buf.data(), nb));
    return buf;
  }
  void restore(const std::vector<char> &buf, void *stream = nullptr) {
    destroy();
    check(hodlr_checkpoint_load(buf.data(), (int64_t)buf.size(), stream, &h_));
    int64_t n = 0;
    std::memcpy(&n, buf.data() + 16, sizeof n);  // the header's N (after magic and two 32-bit fields)
    n_ = n;
    factored_ = true;
  }

  // General form: leaf blocks in the KTree layout (ld, leaf_stride) and
  // per-level factors (set_level).
  void create(int64_t N, int rank, int nrhs_max = 1, int precision = HODLR_PREC_FP64, double refine_tol = 1e-12,
              int residual = HODLR_RESID_FP64_TENSOR, void *stream = nullptr) {
    destroy();
    hodlr_desc d{};
    d.n = N;
    d.leaf = (int32_t)(N >> level_);
    d.levels = level_;
    d.rank = rank;
    d.nrhs_max = nrhs_max;
    d.precision = precision;
    d.residual = residual;
    d.refine_tol = refine_tol;
    d.refine_max_iter = 10;
    d.stream = stream;
    check(hodlr_create(&d, &h_));
    n_ = N;
  }
  void set_leaf_blocks(const double *K, int64_t ld, int64_t leaf_stride) {
    check(hodlr_set_leaf_blocks(h_, K, ld, leaf_stride));
    factored_ = false;
  }
  void set_level(int l, const double *U, int64_t ldu, const double *V, int64_t ldv, const double *s = nullptr) {
    check(hodlr_set_lowrank(h_, l, U, ldu, V, ldv, s));
    factored_ = false;
  }

  void factor() {
    check(hodlr_factor(h_));
    factored_ = true;
  }

  // The reference's HMatrix::solve(b) (src/hmatrix.cc:49-96): B (device,
  // N x nrhs, ldb) is overwritten by the solution.  Factorises on first use.
  hodlr_solve_info solve(double *B, int64_t ldb, int nrhs = 1) {
    if (!factored_) factor();
    hodlr_solve_info info{};
    check(hodlr_solve(h_, B, ldb, nrhs, &info));
    return info;
  }
  hodlr_solve_info solve_transpose(double *B, int64_t ldb, int nrhs = 1) {
    if (!factored_) factor();
    hodlr_solve_info info{};
    check(hodlr_solve_transpose(h_, B, ldb, nrhs, &info));
    return info;
  }
  void matvec(const double *X, int64_t ldx, double *Y, int64_t ldy, int nrhs = 1, bool transpose = false) {
    check(hodlr_matvec(h_, transpose ? 1 : 0, X, ldx, Y, ldy, nrhs));
  }

  void destroy() {
    if (h_) hodlr_destroy(h_);
    h_ = nullptr;
    factored_ = false;
  }
  hodlr_handle handle() const { return h_; }
  int64_t rows() const { return n_; }

 private:
  int level_ = 0;
  int64_t n_ = 0;
  hodlr_handle h_ = nullptr;
  bool factored_ = false;
};

// The reference's LMatrix static kernels (include/lmatrix.hpp:119-169) on
// partitioned column-major device buffers.
struct LMatrix {
  // W = V^T U per partition (gemmRed('t', 'n', 1.0, V, U, 0.0, W)).
  static void gemmRed(int nrow, int nPart, int ncolV, int ncolU, const double *V, int64_t ldv, const double *U,
                      int64_t ldu, double *W, int64_t ldw) {
    check(hodlr_gemm_reduce(nrow, nPart, ncolV, ncolU, V, ldv, U, ldu, W, ldw));
  }
  // W_p = alpha U_p Vb_block(p) + beta W_p (gemmBro('n', 'n', alpha, U, Vb, beta, W)).
  static void gemmBro(int nrow, int nPart, int nBlock, int K, int N, double alpha, const double *U, int64_t ldu,
                      const double *Vb, int64_t ldvb, double beta, double *W, int64_t ldw) {
    check(hodlr_gemm_broadcast(nrow, nPart, nBlock, K, N, alpha, U, ldu, Vb, ldvb, beta, W, ldw));
  }
  // VTu.node_solve(VTd): the capacitance systems of nnode nodes, in place.
  static void node_solve(int nnode, int r, int nrhs, const double *VTu, int64_t ldu, double *VTd, int64_t ldd) {
    check(hodlr_node_solve(nnode, r, nrhs, VTu, ldu, VTd, ldd));
  }
  // LMatrix::node_solve(VTu0, VTu1, VTd0, VTd1, ...) of the SPMD drivers
  // (include/lmatrix.hpp:127-130, src/tasks/node_solve_region.cc:77-97): the
  // (rank0 + rank1)-square systems of siblings with unequal ranks, in place.
  static void node_solve(int nnode, int rank0, int rank1, int nrhs, const double *VTu0, int64_t ldu0,
                         const double *VTu1, int64_t ldu1, double *VTd0, int64_t ldd0, double *VTd1, int64_t ldd1) {
    check(hodlr_node_solve_irregular(nnode, rank0, rank1, nrhs, VTu0, ldu0, VTu1, ldu1, VTd0, ldd0, VTd1, ldd1));
  }
};

// The matrix of the SPMD drivers on one GPU: one uniform subtree per shard
// (its own leaf size, depth, rank and precision) under top levels whose
// nodes couple their children with ranks that may differ (see
// hodlr_tree_create).  Shard j's leaves and bases are set on subtree(j) with
// the HMatrix-style calls; the top levels' bases with set_coupling.
class IrregularTree {
 public:
  IrregularTree(int top_levels, const std::vector<hodlr_desc> &shards, const std::vector<int32_t> &coupling_ranks,
                int nrhs_max = 1, void *stream = nullptr) {
    hodlr_tree_desc d{};
    d.top_levels = top_levels;
    d.subtrees = shards.data();
    d.coupling_rank = coupling_ranks.data();
    d.nrhs_max = nrhs_max;
    d.stream = stream;
    if ((int)shards.size() != (1 << top_levels) || (int)coupling_ranks.size() != 2 * ((1 << top_levels) - 1))
      throw Error(HODLR_ERR_INVALID_ARG, "need 2^T shards and 2 (2^T - 1) coupling ranks");
    check(hodlr_tree_create(&d, &t_));
  }
  IrregularTree(const IrregularTree &) = delete;
  IrregularTree &operator=(const IrregularTree &) = delete;
  ~IrregularTree() {
    if (t_) hodlr_tree_destroy(t_);
  }

  hodlr_handle subtree(int j) const {
    hodlr_handle h = nullptr;
    check(hodlr_tree_subtree(t_, j, &h));
    return h;
  }
  void set_leaf_blocks(int j, const double *K, int64_t ld, int64_t leaf_stride) {
    check(hodlr_set_leaf_blocks(subtree(j), K, ld, leaf_stride));
  }
  void set_level(int j, int l, const double *U, int64_t ldu, const double *V, int64_t ldv,
                 const double *s = nullptr) {
    check(hodlr_set_lowrank(subtree(j), l, U, ldu, V, ldv, s));
  }
  // Child `child` of top node (level, pos): U with its own rank, V with the sibling's.
  void set_coupling(int level, int pos, int child, const double *U, int64_t ldu, const double *V, int64_t ldv) {
    check(hodlr_tree_set_coupling(t_, level, pos, child, U, ldu, V, ldv));
  }
  int64_t rows() const {
    int64_t n = 0;
    check(hodlr_tree_rows(t_, &n, nullptr));
    return n;
  }
  void factor() { check(hodlr_tree_factor(t_)); }
  hodlr_solve_info solve(double *B, int64_t ldb, int nrhs = 1) {
    hodlr_solve_info info{};
    check(hodlr_tree_solve(t_, B, ldb, nrhs, &info));
    return info;
  }
  void matvec(const double *X, int64_t ldx, double *Y, int64_t ldy, int nrhs = 1) {
    check(hodlr_tree_matvec(t_, X, ldx, Y, ldy, nrhs));
  }

 private:
  hodlr_tree t_ = nullptr;
};

}  // namespace hodlr_gb300

#endif  // HODLR_GB300_HPP
