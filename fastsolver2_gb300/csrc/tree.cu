// Irregular HODLR trees: uniform subtrees, each with its own leaf size, depth
// and rank, joined by top levels whose sibling blocks may have unequal ranks.
//
// This is the shape of fastSolver2's SPMD drivers: spmd_driver/solver.cc
// splits the tree into one uniform subtree per shard under spmd_level top
// levels; solver_irregular_part.cc:73-79 gives the first `-heavy` shards a
// leaf ten times larger, and solver_irregular_ranks.cc:99-108 gives the two
// shards ranks rank0 and rank1, their top coupling blocks built with the
// sibling's rank (VMatp, :118-132).  Each top node then solves the
// (r0 + r1)-square system of NodeSolveRegionTask
// (src/tasks/node_solve_region.cc:77-97):
//
//     [ I_r0          V_c1^T U~_c1 ] [eta0]   [ V_c1^T d_c1 ]
//     [ V_c0^T U~_c0  I_r1         ] [eta1] = [ V_c0^T d_c0 ]
//
// for A[c0,c1] = U_c0 V_c1^T (rank r0) and A[c1,c0] = U_c1 V_c0^T (rank r1),
// then d_c0 -= U~_c0 eta0, d_c1 -= U~_c1 eta1.  The subtrees are ordinary
// handles (their leaves, levels and precision are theirs); the top levels run
// in FP64 here: the row reductions and updates of the uniform path on the
// children's rows, and tree_node_kernel for the unequal-rank systems.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace hodlr {

// One top node of an irregular tree.  T0 = V_c0^T X_c0 is r1 x cols (ld r1),
// T1 = V_c1^T X_c1 is r0 x cols (ld r0), both in the reduction scratch; the
// node's LU ((r0+r1)^2, ld r0+r1) and pivots are kept from the factorisation;
// eta is (r0+r1) x cols with ld r0+r1.  anc: the coupling columns of the
// levels above the node on its rows (ranks of its ancestors' blocks, so it
// differs between nodes of one depth).
struct TreeNode {
  long long t0, t1, lu, eta;
  int piv, r0, r1, anc;
};

constexpr int kTreeMaxRank = 64;          // per side
constexpr int kTreeMaxN = 2 * kTreeMaxRank;
constexpr int kTreeChunk = 32;            // right-hand-side columns per pass

// The nodes [node_base, node_base + gridDim.x) of one depth, one CTA each.
// factor: the T blocks hold [ancestor columns | own columns]; S is built from
// the own columns [anc, anc + r), LU-factorised with partial pivoting (the
// pivot is the first entry of largest magnitude, as IDAMAX picks it; the
// column below it is scaled by the pivot's reciprocal, as DGETRF2 does) and
// stored, and the right-hand sides are the anc ancestor columns.  Otherwise
// (solve) the stored LU is loaded and the right-hand sides are nrhs columns.
// The right-hand sides [T1; T0] are solved (row interchanges, unit-lower and
// upper triangular substitution in the order of DGETRS) into eta.
__global__ void __launch_bounds__(256) tree_node_kernel(const TreeNode *nodes, int node_base, const double *red,
                                                        int factor, int nrhs, double *lu, int *ipiv, double *eta,
                                                        DevStatus *st) {
  extern __shared__ double sm[];
  __shared__ int piv[kTreeMaxN];
  const TreeNode nd = nodes[node_base + blockIdx.x];
  const int r0 = nd.r0, r1 = nd.r1, n = r0 + r1, tid = threadIdx.x;
  const int s_col = nd.anc, ncol = factor ? nd.anc : nrhs;
  double *S = sm;           // n x n, ld n
  double *B = sm + n * n;   // n x kTreeChunk, ld n
  const double *T0 = red + nd.t0, *T1 = red + nd.t1;
  double *LU = lu + nd.lu;
  int *gp = ipiv + nd.piv;
  if (factor) {
    for (int e = tid; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      double v = i == j ? 1.0 : 0.0;
      if (i < r0 && j >= r0) v = T1[i + (long long)(s_col + j - r0) * r0];
      else if (i >= r0 && j < r0) v = T0[(i - r0) + (long long)(s_col + j) * r1];
      S[e] = v;
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
      if (tid < 32) {
        double best = -1.0;
        int bi = j;
        for (int i = j + tid; i < n; i += 32) {
          const double v = fabs(S[i + j * n]);
          if (v > best) {
            best = v;
            bi = i;
          }
        }
        for (int off = 16; off; off >>= 1) {
          const double ov = __shfl_down_sync(0xffffffffu, best, off);
          const int oi = __shfl_down_sync(0xffffffffu, bi, off);
          if (ov > best || (ov == best && oi < bi)) {
            best = ov;
            bi = oi;
          }
        }
        if (tid == 0) piv[j] = bi;
      }
      __syncthreads();
      const int p = piv[j];
      if (p != j)
        for (int k = tid; k < n; k += blockDim.x) {
          const double a = S[j + k * n];
          S[j + k * n] = S[p + k * n];
          S[p + k * n] = a;
        }
      __syncthreads();
      const double d = S[j + j * n];
      if (d == 0.0) {
        if (tid == 0) report_error(st, HODLR_ERR_SINGULAR_CAPACITANCE, node_base + blockIdx.x);
      } else {
        const double rinv = 1.0 / d;
        for (int i = j + 1 + tid; i < n; i += blockDim.x) S[i + j * n] *= rinv;
      }
      __syncthreads();
      const int m = n - j - 1;
      for (int e = tid; e < m * m; e += blockDim.x) {
        const int i = j + 1 + e % m, k = j + 1 + e / m;
        S[i + k * n] -= S[i + j * n] * S[j + k * n];
      }
      __syncthreads();
    }
    for (int e = tid; e < n * n; e += blockDim.x) LU[e] = S[e];
    for (int j = tid; j < n; j += blockDim.x) gp[j] = piv[j];
  } else {
    for (int e = tid; e < n * n; e += blockDim.x) S[e] = LU[e];
    for (int j = tid; j < n; j += blockDim.x) piv[j] = gp[j];
  }
  __syncthreads();
  double *E = eta + nd.eta;
  for (int c0 = 0; c0 < ncol; c0 += kTreeChunk) {
    const int cw = min(kTreeChunk, ncol - c0);
    for (int e = tid; e < n * cw; e += blockDim.x) {
      const int i = e % n, c = e / n;
      B[i + c * n] = i < r0 ? T1[i + (long long)(c0 + c) * r0] : T0[(i - r0) + (long long)(c0 + c) * r1];
    }
    __syncthreads();
    if (tid < cw)
      for (int j = 0; j < n; ++j) {
        const int p = piv[j];
        if (p != j) {
          const double a = B[j + tid * n];
          B[j + tid * n] = B[p + tid * n];
          B[p + tid * n] = a;
        }
      }
    __syncthreads();
    for (int j = 0; j + 1 < n; ++j) {  // L y = P b (unit diagonal)
      const int m = n - j - 1;
      for (int e = tid; e < m * cw; e += blockDim.x) {
        const int i = j + 1 + e % m, c = e / m;
        B[i + c * n] -= S[i + j * n] * B[j + c * n];
      }
      __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {  // U x = y
      if (tid < cw) B[j + tid * n] /= S[j + j * n];
      __syncthreads();
      for (int e = tid; e < j * cw; e += blockDim.x) {
        const int i = e % j, c = e / j;
        B[i + c * n] -= S[i + j * n] * B[j + c * n];
      }
      __syncthreads();
    }
    for (int e = tid; e < n * cw; e += blockDim.x) {
      const int i = e % n, c = e / n;
      E[i + (long long)(c0 + c) * n] = B[i + c * n];
    }
    __syncthreads();
  }
}

static size_t tree_node_smem(int nmax) { return sizeof(double) * ((size_t)nmax * nmax + (size_t)nmax * kTreeChunk); }

static cudaError_t launch_tree_nodes(const TreeNode *nodes, int node_base, int count, int nmax, const double *red,
                                     bool factor, int nrhs, double *lu, int *ipiv, double *eta, DevStatus *st,
                                     cudaStream_t s) {
  const size_t bytes = tree_node_smem(nmax);
  cudaError_t e = allow_dyn_smem(tree_node_kernel, bytes);
  if (e != cudaSuccess) return e;
  HODLR_LAUNCH(tree_node_kernel, count, 256, bytes, s, nodes, node_base, red, (int)factor, nrhs, lu, ipiv, eta,
               st);
  return cudaGetLastError();
}

}  // namespace hodlr

using namespace hodlr;

static int tree_err(int code, const std::string &msg) {
  set_last_error(code, msg.c_str());
  return code;
}

#define TCK(expr)                                                                                         \
  do {                                                                                                    \
    cudaError_t e_ = (expr);                                                                              \
    if (e_ != cudaSuccess)                                                                                \
      return tree_err(e_ == cudaErrorMemoryAllocation ? HODLR_ERR_OUT_OF_MEMORY : HODLR_ERR_CUDA,         \
                      std::string(#expr) + ": " + cudaGetErrorString(e_));                                \
  } while (0)

#define TCKS(expr)                 \
  do {                             \
    int s_ = (expr);               \
    if (s_ != HODLR_OK) return s_; \
  } while (0)

struct hodlr_tree_ctx {
  int T = 0, nsub = 0, nnode = 0, kmax = 0, nmax = 0;
  std::vector<hodlr_handle> sub;
  std::vector<long long> n, off;       // subtree rows; first internal row (multiple of 32)
  long long npad = 0, ntot = 0;
  std::vector<int> rk;                 // coupling ranks, 2 per node
  std::vector<int> ucols;              // per subtree: coupling columns of U (all its top levels)
  int wu = 0, wv = 0;
  std::vector<char> coupled;           // per node and child: bases set
  // device: original and transformed coupling bases, V, solve / product buffers
  double *U0 = nullptr, *Ug = nullptr, *Vg = nullptr, *X = nullptr, *Y = nullptr;
  double *red = nullptr, *lu = nullptr, *eta = nullptr, *work = nullptr;
  int *ipiv = nullptr;
  TreeNode *dnodes = nullptr;
  std::vector<TreeNode> nodes;
  DevStatus *dst = nullptr, *hst = nullptr;
  cudaStream_t s = nullptr;
  bool own_stream = false, factored = false;
};

namespace {

// Depth-l ancestor of top leaf j: node index and which child j lies under.
inline int anc_node(int T, int l, int j) { return (1 << l) - 1 + (j >> (T - l)); }
inline int anc_child(int T, int l, int j) { return (j >> (T - 1 - l)) & 1; }

// U / V columns of the levels above depth l on top leaf j.
int ucol(const hodlr_tree_ctx *t, int l, int j) {
  int c = 0;
  for (int a = 0; a < l; ++a) c += t->rk[2 * anc_node(t->T, a, j) + anc_child(t->T, a, j)];
  return c;
}
int vcol(const hodlr_tree_ctx *t, int l, int j) {
  int c = 0;
  for (int a = 0; a < l; ++a) c += t->rk[2 * anc_node(t->T, a, j) + 1 - anc_child(t->T, a, j)];
  return c;
}

// Child h of the depth-l node at position q: its top leaves [j0, j1) and its
// internal rows [row0, row0 + rows).
struct Child {
  int j0, j1;
  long long row0, rows;
};
Child child_of(const hodlr_tree_ctx *t, int l, int q, int h) {
  Child c;
  const int span = 1 << (t->T - 1 - l);
  c.j0 = (2 * q + h) * span;
  c.j1 = c.j0 + span;
  c.row0 = t->off[c.j0];
  c.rows = t->off[c.j1 - 1] + t->n[c.j1 - 1] - c.row0;
  return c;
}

void tree_free(hodlr_tree_ctx *t) {
  for (auto h : t->sub)
    if (h) hodlr_destroy(h);
  t->sub.clear();
  for (void *p : {(void *)t->U0, (void *)t->Ug, (void *)t->Vg, (void *)t->X, (void *)t->Y, (void *)t->red,
                  (void *)t->lu, (void *)t->eta, (void *)t->work, (void *)t->ipiv, (void *)t->dnodes,
                  (void *)t->dst})
    if (p) cudaFree(p);
  if (t->hst) cudaFreeHost(t->hst);
  if (t->own_stream && t->s) cudaStreamDestroy(t->s);
  delete t;
}

int read_status(hodlr_tree_ctx *t, const char *what) {
  TCK(cudaMemcpyAsync(t->hst, t->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, t->s));
  TCK(cudaStreamSynchronize(t->s));
  if (t->hst->code != HODLR_OK) {
    char buf[160];
    snprintf(buf, sizeof buf, "%s: status %d (node %lld)", what, t->hst->code, t->hst->index);
    return tree_err(t->hst->code, buf);
  }
  return HODLR_OK;
}

// T blocks of every node of depth l: T0 = V_c0^T X_c0(:, 0:C0), T1 = V_c1^T
// X_c1(:, 0:C1) with C_h = xcols(node, h) columns of X (leading dimension npad).
template <typename F>
int reduce_level(hodlr_tree_ctx *t, int l, const double *X, F xcols) {
  for (int q = 0; q < (1 << l); ++q) {
    const int p = (1 << l) - 1 + q;
    const TreeNode &nd = t->nodes[p];
    for (int h = 0; h < 2; ++h) {
      const Child c = child_of(t, l, q, h);
      const int rv = t->rk[2 * p + 1 - h];  // V_c has the sibling's rank
      const double *V = t->Vg + c.row0 + (long long)vcol(t, l, c.j0) * t->npad;
      TCK(launch_reduce_tn<double>(V, t->npad, X + c.row0, t->npad, c.rows, 1, rv, xcols(nd, h), t->red + (h ? nd.t1 : nd.t0),
                                   t->work, nullptr, t->s, t->dst));
    }
  }
  return HODLR_OK;
}

// X_c(:, 0:ncol) -= U~_c(own columns of depth l) eta_h for both children of
// every node of depth l (Ubase: the transformed bases, leading dimension npad;
// ncol < 0: each node's ancestor columns).
int update_level(hodlr_tree_ctx *t, int l, double *X, int ncol_arg, const double *Ubase, double alpha) {
  for (int q = 0; q < (1 << l); ++q) {
    const int p = (1 << l) - 1 + q;
    const TreeNode &nd = t->nodes[p];
    const int n = nd.r0 + nd.r1;
    const int ncol = ncol_arg < 0 ? nd.anc : ncol_arg;
    if (ncol == 0) continue;
    for (int h = 0; h < 2; ++h) {
      const Child c = child_of(t, l, q, h);
      UpdateArgs ua{};
      ua.A = Ubase + c.row0 + (long long)ucol(t, l, c.j0) * t->npad;
      ua.lda = t->npad;
      ua.B = t->eta + nd.eta + (h ? nd.r0 : 0);
      ua.ldb = n;
      ua.C = X + c.row0;
      ua.ldc = t->npad;
      ua.M = (int)c.rows;
      ua.N = ncol;
      ua.K = h ? nd.r1 : nd.r0;
      ua.nbatch = 1;
      ua.alpha = alpha;
      TCK(launch_update_nn<double>(ua, t->s, t->dst));
    }
  }
  return HODLR_OK;
}

}  // namespace

extern "C" {

int hodlr_tree_create(const hodlr_tree_desc *d, hodlr_tree *out) {
  if (!d || !out || !d->subtrees || !d->coupling_rank) return tree_err(HODLR_ERR_INVALID_ARG, "tree: null argument");
  *out = nullptr;
  if (d->top_levels < 1 || d->top_levels > 7 || d->nrhs_max < 1)
    return tree_err(HODLR_ERR_INVALID_ARG, "tree: need 1 <= top_levels <= 7 and nrhs_max >= 1");
  auto *t = new hodlr_tree_ctx();
  t->T = d->top_levels;
  t->nsub = 1 << t->T;
  t->nnode = t->nsub - 1;
  t->kmax = d->nrhs_max;
  t->rk.assign(d->coupling_rank, d->coupling_rank + 2 * t->nnode);
  for (int v : t->rk)
    if (v < 1 || v > kTreeMaxRank) {
      tree_free(t);
      return tree_err(HODLR_ERR_INVALID_ARG, "tree: coupling ranks must be 1..64");
    }
  t->n.resize(t->nsub);
  t->off.resize(t->nsub);
  t->ucols.resize(t->nsub);
  for (int j = 0; j < t->nsub; ++j) {
    t->n[j] = d->subtrees[j].n;
    t->off[j] = t->npad;
    t->npad += (t->n[j] + 31) / 32 * 32;
    t->ntot += t->n[j];
    t->ucols[j] = ucol(t, t->T, j);
    t->wu = std::max(t->wu, t->ucols[j]);
    t->wv = std::max(t->wv, vcol(t, t->T, j));
  }
  if (d->stream) {
    t->s = (cudaStream_t)d->stream;
  } else {
    if (cudaStreamCreateWithFlags(&t->s, cudaStreamNonBlocking) != cudaSuccess) {
      tree_free(t);
      return tree_err(HODLR_ERR_CUDA, "tree: stream");
    }
    t->own_stream = true;
  }
  for (int j = 0; j < t->nsub; ++j) {
    hodlr_desc sd = d->subtrees[j];
    sd.nrhs_max = std::max(t->kmax, t->ucols[j]);
    sd.stream = t->s;
    hodlr_handle h = nullptr;
    const int rc = hodlr_create(&sd, &h);
    if (rc != HODLR_OK) {
      const std::string msg = std::string("tree: subtree ") + std::to_string(j) + ": " + hodlr_last_error_string();
      tree_free(t);
      return tree_err(rc, msg);
    }
    t->sub.push_back(h);
  }
  // node table: reduction blocks sized for max(factor columns, nrhs_max)
  long long red = 0, lus = 0, etas = 0;
  int pivs = 0;
  size_t work = 0;
  t->nodes.resize(t->nnode);
  for (int l = 0; l < t->T; ++l)
    for (int q = 0; q < (1 << l); ++q) {
      const int p = (1 << l) - 1 + q;
      TreeNode &nd = t->nodes[p];
      nd.r0 = t->rk[2 * p];
      nd.r1 = t->rk[2 * p + 1];
      const int nn = nd.r0 + nd.r1;
      const int a = ucol(t, l, child_of(t, l, q, 0).j0);  // ancestor columns (both children)
      nd.anc = a;
      const int c0 = std::max(a + nd.r0, t->kmax), c1 = std::max(a + nd.r1, t->kmax);
      nd.t0 = red;
      red += (long long)nd.r1 * c0;
      nd.t1 = red;
      red += (long long)nd.r0 * c1;
      nd.lu = lus;
      lus += (long long)nn * nn;
      nd.eta = etas;
      etas += (long long)nn * std::max(a, t->kmax);
      nd.piv = pivs;
      pivs += nn;
      t->nmax = std::max(t->nmax, nn);
      for (int h = 0; h < 2; ++h) {  // every column count a reduction of this child is given
        const Child c = child_of(t, l, q, h);
        const int rv = h ? nd.r0 : nd.r1;
        for (int C = 1; C <= std::max(c0, c1); ++C)
          work = std::max(work, reduce_workspace_doubles(c.rows, 1, rv, C, 8));
      }
    }
  t->coupled.assign(2 * t->nnode, 0);
  cudaError_t e = cudaSuccess;
  auto alloc = [&](auto **p, size_t count) {
    if (e == cudaSuccess) e = cudaMalloc((void **)p, sizeof(**p) * std::max<size_t>(count, 1));
  };
  alloc(&t->U0, (size_t)t->npad * t->wu);
  alloc(&t->Ug, (size_t)t->npad * t->wu);
  alloc(&t->Vg, (size_t)t->npad * t->wv);
  alloc(&t->X, (size_t)t->npad * t->kmax);
  alloc(&t->Y, (size_t)t->npad * t->kmax);
  alloc(&t->red, (size_t)red);
  alloc(&t->lu, (size_t)lus);
  alloc(&t->eta, (size_t)etas);
  alloc(&t->work, work);
  alloc(&t->ipiv, (size_t)pivs);
  alloc(&t->dnodes, (size_t)t->nnode);
  alloc(&t->dst, 1);
  if (e == cudaSuccess) e = cudaMallocHost((void **)&t->hst, sizeof(DevStatus));
  // padding rows stay zero in every buffer
  for (double *p : {t->U0, t->Ug, t->X, t->Y})
    if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, sizeof(double) * t->npad * (p == t->X || p == t->Y ? t->kmax : t->wu), t->s);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->Vg, 0, sizeof(double) * t->npad * std::max(t->wv, 1), t->s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(t->dnodes, t->nodes.data(), sizeof(TreeNode) * t->nnode, cudaMemcpyHostToDevice, t->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(t->s);
  if (e != cudaSuccess) {
    tree_free(t);
    return tree_err(e == cudaErrorMemoryAllocation ? HODLR_ERR_OUT_OF_MEMORY : HODLR_ERR_CUDA,
                    std::string("tree: ") + cudaGetErrorString(e));
  }
  *out = t;
  return HODLR_OK;
}

int hodlr_tree_destroy(hodlr_tree t) {
  if (!t) return HODLR_OK;
  cudaStreamSynchronize(t->s);
  tree_free(t);
  return HODLR_OK;
}

int hodlr_tree_subtree(hodlr_tree t, int j, hodlr_handle *out) {
  if (!t || !out || j < 0 || j >= t->nsub) return tree_err(HODLR_ERR_INVALID_ARG, "tree_subtree: bad arguments");
  *out = t->sub[j];
  t->factored = false;
  return HODLR_OK;
}

int hodlr_tree_rows(hodlr_tree t, int64_t *n, int64_t *row_offsets) {
  if (!t || !n) return tree_err(HODLR_ERR_INVALID_ARG, "tree_rows: null argument");
  *n = t->ntot;
  if (row_offsets) {
    long long o = 0;
    for (int j = 0; j < t->nsub; ++j) {
      row_offsets[j] = o;
      o += t->n[j];
    }
    row_offsets[t->nsub] = o;
  }
  return HODLR_OK;
}

int hodlr_tree_set_coupling(hodlr_tree t, int level, int pos, int child, const double *U, int64_t ldu,
                            const double *V, int64_t ldv) {
  if (!t || !U || !V || level < 0 || level >= t->T || pos < 0 || pos >= (1 << level) || (child != 0 && child != 1))
    return tree_err(HODLR_ERR_INVALID_ARG, "tree_set_coupling: bad arguments");
  const int p = (1 << level) - 1 + pos;
  const Child c = child_of(t, level, pos, child);
  long long rows = 0;
  for (int j = c.j0; j < c.j1; ++j) rows += t->n[j];
  if (ldu < rows || ldv < rows) return tree_err(HODLR_ERR_INVALID_ARG, "tree_set_coupling: ld < child rows");
  const int ru = t->rk[2 * p + child], rv = t->rk[2 * p + 1 - child];
  const int uc = ucol(t, level, c.j0), vc = vcol(t, level, c.j0);
  long long src = 0;  // the caller's rows are the child's rows, packed
  for (int j = c.j0; j < c.j1; ++j) {
    TCK(cudaMemcpy2DAsync(t->U0 + t->off[j] + (long long)uc * t->npad, sizeof(double) * t->npad, U + src,
                          sizeof(double) * ldu, sizeof(double) * t->n[j], ru, cudaMemcpyDefault, t->s));
    TCK(cudaMemcpy2DAsync(t->Vg + t->off[j] + (long long)vc * t->npad, sizeof(double) * t->npad, V + src,
                          sizeof(double) * ldv, sizeof(double) * t->n[j], rv, cudaMemcpyDefault, t->s));
    src += t->n[j];
  }
  TCK(cudaStreamSynchronize(t->s));
  t->coupled[2 * p + child] = 1;
  t->factored = false;
  return HODLR_OK;
}

int hodlr_tree_factor(hodlr_tree t) {
  if (!t) return tree_err(HODLR_ERR_INVALID_ARG, "tree_factor: null argument");
  for (char c : t->coupled)
    if (!c) return tree_err(HODLR_ERR_NOT_FACTORED, "tree_factor: coupling bases not set");
  t->factored = false;
  for (int j = 0; j < t->nsub; ++j) {
    const int rc = hodlr_factor(t->sub[j]);
    if (rc != HODLR_OK)
      return tree_err(rc, std::string("tree_factor: subtree ") + std::to_string(j) + ": " + hodlr_last_error_string());
  }
  TCK(cudaMemsetAsync(t->dst, 0, sizeof(DevStatus), t->s));
  TCK(cudaMemcpyAsync(t->Ug, t->U0, sizeof(double) * t->npad * t->wu, cudaMemcpyDeviceToDevice, t->s));
  // U~ = A_j^{-1} U on every subtree (all of its coupling columns at once)
  for (int j = 0; j < t->nsub; ++j) {
    const int rc = hodlr_solve(t->sub[j], t->Ug + t->off[j], t->npad, t->ucols[j], nullptr);
    if (rc != HODLR_OK)
      return tree_err(rc, std::string("tree_factor: subtree ") + std::to_string(j) + ": " + hodlr_last_error_string());
  }
  // top levels, deepest first: S from the children's own columns, then the
  // ancestors' columns updated with the solved system
  for (int l = t->T - 1; l >= 0; --l) {
    const int base = (1 << l) - 1;
    TCKS(reduce_level(t, l, t->Ug, [&](const TreeNode &nd, int h) { return nd.anc + (h ? nd.r1 : nd.r0); }));
    TCK(launch_tree_nodes(t->dnodes, base, 1 << l, t->nmax, t->red, true, 0, t->lu, t->ipiv, t->eta, t->dst, t->s));
    TCKS(update_level(t, l, t->Ug, -1, t->Ug, -1.0));
  }
  TCKS(read_status(t, "tree_factor"));
  t->factored = true;
  return HODLR_OK;
}

int hodlr_tree_solve(hodlr_tree t, double *B, int64_t ldb, int nrhs, hodlr_solve_info *info) {
  if (!t || !B) return tree_err(HODLR_ERR_INVALID_ARG, "tree_solve: null argument");
  if (!t->factored) return tree_err(HODLR_ERR_NOT_FACTORED, "tree_solve: call hodlr_tree_factor first");
  if (nrhs < 1 || nrhs > t->kmax || ldb < t->ntot) return tree_err(HODLR_ERR_INVALID_ARG, "tree_solve: bad nrhs / ldb");
  if (info) *info = hodlr_solve_info{0, 0, -1, -1.0};
  long long src = 0;
  for (int j = 0; j < t->nsub; ++j) {
    TCK(cudaMemcpy2DAsync(t->X + t->off[j], sizeof(double) * t->npad, B + src, sizeof(double) * ldb,
                          sizeof(double) * t->n[j], nrhs, cudaMemcpyDeviceToDevice, t->s));
    src += t->n[j];
  }
  for (int j = 0; j < t->nsub; ++j) {
    hodlr_solve_info si{};
    const int rc = hodlr_solve(t->sub[j], t->X + t->off[j], t->npad, nrhs, &si);
    if (rc != HODLR_OK)
      return tree_err(rc, std::string("tree_solve: subtree ") + std::to_string(j) + ": " + hodlr_last_error_string());
    if (info) {
      info->iterations = std::max(info->iterations, si.iterations);
      info->rel_residual = std::max(info->rel_residual, si.rel_residual);
    }
  }
  TCK(cudaMemsetAsync(t->dst, 0, sizeof(DevStatus), t->s));
  for (int l = t->T - 1; l >= 0; --l) {
    TCKS(reduce_level(t, l, t->X, [&](const TreeNode &, int) { return nrhs; }));
    TCK(launch_tree_nodes(t->dnodes, (1 << l) - 1, 1 << l, t->nmax, t->red, false, nrhs, t->lu, t->ipiv, t->eta,
                          t->dst, t->s));
    TCKS(update_level(t, l, t->X, nrhs, t->Ug, -1.0));
  }
  src = 0;
  for (int j = 0; j < t->nsub; ++j) {
    TCK(cudaMemcpy2DAsync(B + src, sizeof(double) * ldb, t->X + t->off[j], sizeof(double) * t->npad,
                          sizeof(double) * t->n[j], nrhs, cudaMemcpyDeviceToDevice, t->s));
    src += t->n[j];
  }
  TCKS(read_status(t, "tree_solve"));
  return HODLR_OK;
}

int hodlr_tree_matvec(hodlr_tree t, const double *X, int64_t ldx, double *Y, int64_t ldy, int nrhs) {
  if (!t || !X || !Y) return tree_err(HODLR_ERR_INVALID_ARG, "tree_matvec: null argument");
  if (nrhs < 1 || nrhs > t->kmax || ldx < t->ntot || ldy < t->ntot)
    return tree_err(HODLR_ERR_INVALID_ARG, "tree_matvec: bad nrhs / ld");
  for (char c : t->coupled)
    if (!c) return tree_err(HODLR_ERR_NOT_FACTORED, "tree_matvec: coupling bases not set");
  long long src = 0;
  for (int j = 0; j < t->nsub; ++j) {
    TCK(cudaMemcpy2DAsync(t->X + t->off[j], sizeof(double) * t->npad, X + src, sizeof(double) * ldx,
                          sizeof(double) * t->n[j], nrhs, cudaMemcpyDeviceToDevice, t->s));
    src += t->n[j];
  }
  for (int j = 0; j < t->nsub; ++j) {
    const int rc = hodlr_matvec(t->sub[j], 0, t->X + t->off[j], t->npad, t->Y + t->off[j], t->npad, nrhs);
    if (rc != HODLR_OK)
      return tree_err(rc, std::string("tree_matvec: subtree ") + std::to_string(j) + ": " + hodlr_last_error_string());
  }
  TCK(cudaMemsetAsync(t->dst, 0, sizeof(DevStatus), t->s));
  // A[c0,c1] X_c1 = U_c0 (V_c1^T X_c1): the T blocks double as eta here
  for (int l = 0; l < t->T; ++l) {
    TCKS(reduce_level(t, l, t->X, [&](const TreeNode &, int) { return nrhs; }));
    for (int q = 0; q < (1 << l); ++q) {
      const int p = (1 << l) - 1 + q;
      const TreeNode &nd = t->nodes[p];
      for (int h = 0; h < 2; ++h) {
        const Child c = child_of(t, l, q, h);
        UpdateArgs ua{};
        ua.A = t->U0 + c.row0 + (long long)ucol(t, l, c.j0) * t->npad;
        ua.lda = t->npad;
        ua.B = t->red + (h ? nd.t0 : nd.t1);  // V_sib^T X_sib
        ua.ldb = h ? nd.r1 : nd.r0;
        ua.C = t->Y + c.row0;
        ua.ldc = t->npad;
        ua.M = (int)c.rows;
        ua.N = nrhs;
        ua.K = h ? nd.r1 : nd.r0;
        ua.nbatch = 1;
        ua.alpha = 1.0;
        TCK(launch_update_nn<double>(ua, t->s, t->dst));
      }
    }
  }
  src = 0;
  for (int j = 0; j < t->nsub; ++j) {
    TCK(cudaMemcpy2DAsync(Y + src, sizeof(double) * ldy, t->Y + t->off[j], sizeof(double) * t->npad,
                          sizeof(double) * t->n[j], nrhs, cudaMemcpyDeviceToDevice, t->s));
    src += t->n[j];
  }
  return read_status(t, "tree_matvec");
}

// NodeSolveRegionTask (src/tasks/node_solve_region.cc:77-97) for nnode nodes
// at once, through the same kernel as the tree's top levels.
int hodlr_node_solve_irregular(int nnode, int r0, int r1, int nrhs, const double *VTu0, int64_t ldu0,
                               const double *VTu1, int64_t ldu1, double *VTd0, int64_t ldd0, double *VTd1,
                               int64_t ldd1) {
  if (!VTu0 || !VTu1 || !VTd0 || !VTd1 || nnode < 1 || r0 < 1 || r1 < 1 || r0 > kTreeMaxRank ||
      r1 > kTreeMaxRank || nrhs < 1 || ldu0 < (int64_t)nnode * r1 || ldd0 < (int64_t)nnode * r1 ||
      ldu1 < (int64_t)nnode * r0 || ldd1 < (int64_t)nnode * r0)
    return tree_err(HODLR_ERR_INVALID_ARG, "node_solve_irregular: bad arguments");
  const int n = r0 + r1;
  std::vector<TreeNode> nodes(nnode);
  long long red = 0;
  for (int p = 0; p < nnode; ++p) {  // T0 = [VTd0 | VTu0] (r1 rows), T1 = [VTd1 | VTu1] (r0 rows)
    nodes[p].t0 = red;
    red += (long long)r1 * (nrhs + r0);
    nodes[p].t1 = red;
    red += (long long)r0 * (nrhs + r1);
    nodes[p].lu = (long long)p * n * n;
    nodes[p].eta = (long long)p * n * nrhs;
    nodes[p].piv = p * n;
    nodes[p].r0 = r0;
    nodes[p].r1 = r1;
    nodes[p].anc = nrhs;  // the right-hand sides take the ancestor columns' place
  }
  double *dred = nullptr, *dlu = nullptr, *deta = nullptr;
  int *dpiv = nullptr;
  TreeNode *dn = nullptr;
  DevStatus *dst = nullptr;
  cudaError_t e = cudaMalloc(&dred, sizeof(double) * red);
  if (e == cudaSuccess) e = cudaMalloc(&dlu, sizeof(double) * nnode * n * n);
  if (e == cudaSuccess) e = cudaMalloc(&deta, sizeof(double) * nnode * n * nrhs);
  if (e == cudaSuccess) e = cudaMalloc(&dpiv, sizeof(int) * nnode * n);
  if (e == cudaSuccess) e = cudaMalloc(&dn, sizeof(TreeNode) * nnode);
  if (e == cudaSuccess) e = cudaMalloc(&dst, sizeof(DevStatus));
  if (e == cudaSuccess) e = cudaMemsetAsync(dst, 0, sizeof(DevStatus), 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dn, nodes.data(), sizeof(TreeNode) * nnode, cudaMemcpyHostToDevice, 0);
  for (int p = 0; p < nnode && e == cudaSuccess; ++p) {
    double *t0 = dred + nodes[p].t0, *t1 = dred + nodes[p].t1;
    e = cudaMemcpy2DAsync(t0, sizeof(double) * r1, VTd0 + (long long)p * r1, sizeof(double) * ldd0,
                          sizeof(double) * r1, nrhs, cudaMemcpyDeviceToDevice, 0);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(t0 + (long long)r1 * nrhs, sizeof(double) * r1, VTu0 + (long long)p * r1,
                            sizeof(double) * ldu0, sizeof(double) * r1, r0, cudaMemcpyDeviceToDevice, 0);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(t1, sizeof(double) * r0, VTd1 + (long long)p * r0, sizeof(double) * ldd1,
                            sizeof(double) * r0, nrhs, cudaMemcpyDeviceToDevice, 0);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(t1 + (long long)r0 * nrhs, sizeof(double) * r0, VTu1 + (long long)p * r0,
                            sizeof(double) * ldu1, sizeof(double) * r0, r1, cudaMemcpyDeviceToDevice, 0);
  }
  if (e == cudaSuccess) e = launch_tree_nodes(dn, 0, nnode, n, dred, true, 0, dlu, dpiv, deta, dst, 0);
  for (int p = 0; p < nnode && e == cudaSuccess; ++p) {  // eta rows [0, r0) -> VTd1, [r0, n) -> VTd0
    const double *ep = deta + nodes[p].eta;
    e = cudaMemcpy2DAsync(VTd1 + (long long)p * r0, sizeof(double) * ldd1, ep, sizeof(double) * n,
                          sizeof(double) * r0, nrhs, cudaMemcpyDeviceToDevice, 0);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(VTd0 + (long long)p * r1, sizeof(double) * ldd0, ep + r0, sizeof(double) * n,
                            sizeof(double) * r1, nrhs, cudaMemcpyDeviceToDevice, 0);
  }
  DevStatus hs{};
  if (e == cudaSuccess) e = cudaMemcpy(&hs, dst, sizeof(DevStatus), cudaMemcpyDeviceToHost);
  for (void *q : {(void *)dred, (void *)dlu, (void *)deta, (void *)dpiv, (void *)dn, (void *)dst})
    if (q) cudaFree(q);
  if (e != cudaSuccess)
    return tree_err(e == cudaErrorMemoryAllocation ? HODLR_ERR_OUT_OF_MEMORY : HODLR_ERR_CUDA,
                    std::string("node_solve_irregular: ") + cudaGetErrorString(e));
  if (hs.code) return tree_err(hs.code, "node_solve_irregular: singular system");
  return HODLR_OK;
}

}  // extern "C"
