// C ABI of the GB300 HODLR solver: handle life cycle, the factor / solve
// sweeps (one launch per kernel per tree depth, captured in CUDA graphs),
// mixed-precision iterative refinement, the transpose solve / adjoint sweep,
// and the drop-in for fastSolver2's raw-pointer hsolve.
//
// Device layout of a handle (all column-major):
//   D      [nleaf][m][m]   FP64 leaf blocks                (KTree region)
//   U, V   [L][n][r]       FP64 per-level factors, ld n    (UTree chunks / VTree)
//   s      [L][r]          FP64 singular-value scalings
//   LU     [nleaf][m][m]   leaf LU factors (FP64, or FP32 in the mixed mode)
//   ipiv   [nleaf][m]      1-based leaf pivots
//   Ut     n x (L*r)       transformed bases Utilde^(l) = A_c^{-1} U^(l)_c, ld n
//   capLU  [2^L-1][2r][2r] FP64 capacitance LU of every node, node id 2^l-1+p
// Level l's U/V/Ut block is the column range [l*r, (l+1)*r) of an n x L*r
// matrix, i.e. the UTree column layout of the reference (src/tree.cc:61-73)
// without the right-hand-side columns.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "kernels.cuh"
#include "ozaki.cuh"
#include "resid_emul.cuh"

namespace hodlr {
static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

cudaError_t allow_max_dyn_smem(const void *func) {
  static std::mutex mu;
  static std::set<std::pair<const void *, int>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (done.count({func, dev})) return cudaSuccess;
  cudaFuncAttributes fa;
  int optin = 0;
  e = cudaFuncGetAttributes(&fa, func);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  if (e == cudaSuccess) done.insert({func, dev});
  return e;
}
bool debug_sync() {
  static const bool on = [] {
    const char *v = getenv("HODLR_DEBUG_SYNC");
    return v && *v && *v != '0';
  }();
  return on;
}
void debug_after_launch(const char *name, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cs);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && cs == cudaStreamCaptureStatusNone) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) fprintf(stderr, "hodlr: kernel %s: %s\n", name, cudaGetErrorString(e));
}
}  // namespace hodlr

using namespace hodlr;

static thread_local std::string g_err;

static int set_err(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

namespace hodlr {
int set_last_error(int code, const char *msg) { return set_err(code, msg); }
}  // namespace hodlr

#define CK(expr)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (expr);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return set_err(e_ == cudaErrorMemoryAllocation ? HODLR_ERR_OUT_OF_MEMORY : HODLR_ERR_CUDA, \
                     std::string(#expr) + ": " + cudaGetErrorString(e_));                     \
  } while (0)

#define CKS(expr)                  \
  do {                             \
    int s_ = (expr);               \
    if (s_ != HODLR_OK) return s_; \
  } while (0)

// Optional per-phase device timing: CUDA events around every launch of a
// phase (event record nodes inside captured graphs), summed after each call.
struct PhaseRec {
  int phase;
  cudaEvent_t a, b;
};

struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;
  std::vector<PhaseRec> recs;
};

static void destroy_recs(std::vector<PhaseRec> &v) {
  for (auto &p : v) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  v.clear();
}

struct hodlr_ctx {
  hodlr_desc d{};
  long long n = 0;
  int m = 0, L = 0, r = 0, nleaf = 0, nnode = 0, kmax = 0;
  bool mixed = false;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  // inputs
  double *D = nullptr, *U = nullptr, *V = nullptr, *s = nullptr;
  bool has_D = false;
  std::vector<char> has_level;
  // factorisation
  double *LU = nullptr, *Ut = nullptr;
  float *LU32 = nullptr, *V32 = nullptr, *Ut32 = nullptr;
  int *ipiv = nullptr;
  double *capLU = nullptr;
  int *cap_ipiv = nullptr;
  double *Sinv = nullptr;     // [nnode][2r][2r] FP64 capacitance inverses
  float2 *Sinv2 = nullptr;    // their double-word split (unused by the sweeps)
  float *Sinv32 = nullptr;    // mixed mode: FP32 inverses (from the FP64-factored systems)
  double *Dinv = nullptr;     // [nleaf][m][m] leaf inverses (FP64 mode)
  float *Dinv32 = nullptr;    // (mixed mode)
  bool factored = false;
  // workspaces
  double *Tbuf = nullptr, *Wbuf = nullptr, *eta = nullptr, *red = nullptr;
  float *eta32 = nullptr;   // mixed: capacitance solutions rounded for the FP32 updates
  float *Tbuf32 = nullptr;  // mixed: FP32 reductions V^T X of the sweeps
  double *X64 = nullptr, *R64 = nullptr, *B64 = nullptr, *norms = nullptr, *nwork = nullptr;
  float *X32 = nullptr;
  // double-word (hi, lo) copies for the emulated FP64 residual (mixed mode)
  float2 *D2 = nullptr, *U2 = nullptr, *V2 = nullptr, *X2 = nullptr, *R2 = nullptr, *T2 = nullptr;
  bool emulated = false;
  // tensor-core mode: D2 / U2 / V2 serve only the transposed solves, so they
  // are made by the first transposed solve after the inputs change
  bool dw_stale = false;
  // tensor-core residual (HODLR_RESID_FP64_TENSOR): digit slices of D (row
  // scaled), U (row scaled), V (64-row chunks), the iterate X and the
  // coupling blocks T', with their power-of-two exponents
  bool oz = false;
  // the leaf and update products in one tcgen05 pass (oz_tc.cu); Tsl / Texp
  // then hold every level's T' digits one level after another
  bool oz_tc = false;
  double *Tall = nullptr, *Tpart = nullptr;  // every level's V^T X blocks, and their range partials
  __nv_bfloat16 *Dsl = nullptr, *Usl = nullptr, *Vsl = nullptr, *Xsl = nullptr, *Tsl = nullptr;
  int *Dexp = nullptr, *Uexp = nullptr, *Vexp = nullptr, *Xexp = nullptr, *Texp = nullptr;
  size_t tbuf_elems = 0, eta_elems = 0, red_elems = 0;
  DevStatus *dst = nullptr, *hst = nullptr;
  // timing
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // set-time preparation on a side stream (hodlr_set_leaf_blocks /
  // hodlr_set_lowrank): pst, the copy-done event, one prepared event per input
  // (leaf blocks, then level l at 1 + l), and the last one enqueued
  cudaStream_t pst = nullptr;
  cudaStream_t cst = nullptr;  // captures the body of the refinement loop's conditional graph node
  // HODLR_FLAG_STREAM_INPUTS: per level, the pinned host source of a V whose
  // copy waits for the next factorisation (nullptr: V is on the device); the
  // factorisation copies them deepest level first on the side stream, level l
  // signalling vready[l], while the sweep runs
  std::vector<const double *> vsrc;
  std::vector<int64_t> vsrc_ld;
  std::vector<cudaEvent_t> vready, vcopied;
  cudaEvent_t vfork = nullptr;
  cudaStream_t vcs = nullptr;  // the streamed V copies (the side stream prepares each level after its copy)
  std::vector<const double *> sv_captured;  // the sources the streamed factor graphs copy from
  cudaEvent_t pcopy = nullptr, plast = nullptr;
  std::vector<cudaEvent_t> pready;
  // mixed mode: the leaf LU (+ inverses) started on the side stream as soon
  // as the leaf blocks are set, its status in dst_leaf; the next factorisation
  // skips its own leaf LU and takes over that status
  DevStatus *dst_leaf = nullptr;
  bool leaves_prefactored = false;
  // mixed mode, leaf 128: the factorisation forms only the leaf inverses the
  // sweeps apply; LU32 / ipiv are formed on request (ensure_leaf_lu)
  bool lu_stale = false;
  float factor_ms = 0.f, solve_ms = 0.f;
  // graphs
  bool use_graphs = true;
  int factor_runs = 0;
  GraphEntry factor_graph;
  int factor_sv_runs = 0, factor_sv_nl_runs = 0;  // with the V copies streamed in (HODLR_FLAG_STREAM_INPUTS)
  GraphEntry factor_sv_graph, factor_sv_nl_graph;
  int factor_nl_runs = 0;  // the factorisation without its leaf LU (leaves_prefactored)
  GraphEntry factor_nl_graph;
  std::map<std::tuple<const double *, long long, int, int>, GraphEntry> solve_graphs;
  std::map<std::tuple<const double *, long long, int, int>, int> solve_runs;
  std::vector<void *> allocs;
  // phase profiling
  bool profile = false;
  std::vector<PhaseRec> *recs = nullptr;     // where launches record, or null
  std::vector<PhaseRec> *last_recs = nullptr;
  bool last_eager = false;
  std::vector<PhaseRec> eager_recs;
  double phase_ms[HODLR_NUM_PHASES] = {};
  long long phase_n[HODLR_NUM_PHASES] = {};

  template <typename T> T *alloc(size_t count, cudaError_t &err) {
    void *p = nullptr;
    if (count == 0) count = 1;
    err = cudaMalloc(&p, count * sizeof(T));
    if (err == cudaSuccess) allocs.push_back(p);
    return static_cast<T *>(p);
  }
  double *Ulev(int l) const { return U + (long long)l * n * r; }
  double *Vlev(int l) const { return V + (long long)l * n * r; }
  double *slev(int l) const { return s + (long long)l * r; }

  // Level geometry.  Level l = 0 .. L-1 counts from the root of the tallest
  // tree.  One tree: 2^(l+1) child blocks of n / 2^(l+1) rows.  A forest (the
  // systems of a ragged batch that share leaf size and rank, stacked in order
  // of decreasing size) has, at level l, the child blocks of every tree tall
  // enough to have that level: lev_nb[l] blocks of lev_rows[l] rows covering
  // the first lev_nb[l] * lev_rows[l] rows; its nodes are numbered from
  // lev_base[l].  Trees of different depth meet a level at the same height
  // above the leaves, so their blocks there have the same size.
  std::vector<int> lev_nb, lev_base;
  std::vector<long long> lev_rows;
  int nb(int l) const { return lev_nb[l]; }
  long long rows(int l) const { return lev_rows[l]; }
  int nodes(int l) const { return lev_nb[l] / 2; }
  int node_base(int l) const { return lev_base[l]; }
  // systems of a forest (one for a plain handle): leaf offsets, for the
  // per-system residual norms of the refinement test
  int nsys = 1;
  int *seg_leaf = nullptr;  // device [nsys + 1]
  bool forest = false;
  double *sfold = nullptr;  // forest: device copy of one level's s, folded into V
  Tuning tune;              // launch shapes of the tunable kernels (hodlr_autotune)
};

static void clear_sv_graphs(hodlr_ctx *h) {
  for (GraphEntry *g : {&h->factor_sv_graph, &h->factor_sv_nl_graph}) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    destroy_recs(g->recs);
    *g = GraphEntry();
  }
  h->factor_sv_runs = h->factor_sv_nl_runs = 0;
  h->sv_captured.clear();
}

static void clear_graphs(hodlr_ctx *h) {
  for (auto &g : h->solve_graphs) {
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    destroy_recs(g.second.recs);
  }
  h->solve_graphs.clear();
  h->solve_runs.clear();
  if (h->factor_graph.exec) cudaGraphExecDestroy(h->factor_graph.exec);
  destroy_recs(h->factor_graph.recs);
  h->factor_graph = GraphEntry();
  h->factor_runs = 0;
  if (h->factor_nl_graph.exec) cudaGraphExecDestroy(h->factor_nl_graph.exec);
  destroy_recs(h->factor_nl_graph.recs);
  h->factor_nl_graph = GraphEntry();
  h->factor_nl_runs = 0;
  clear_sv_graphs(h);
  h->last_recs = nullptr;
}

// Inside stream capture a plain cudaEventRecord only orders streams; the
// External flag makes it an event-record node that records on every replay.
static void record_timing_event(cudaEvent_t e, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cs);
  if (cs == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
  else
    cudaEventRecord(e, s);
}

struct PhaseScope {
  hodlr_ctx *h;
  int ph;
  cudaEvent_t a = nullptr;
  PhaseScope(hodlr_ctx *h_, int ph_) : h(h_), ph(ph_) {
    if (h->profile && h->recs && cudaEventCreate(&a) == cudaSuccess) record_timing_event(a, h->st);
  }
  ~PhaseScope() {
    if (!a) return;
    cudaEvent_t b;
    if (cudaEventCreate(&b) != cudaSuccess) {
      cudaEventDestroy(a);
      return;
    }
    record_timing_event(b, h->st);
    h->recs->push_back({ph, a, b});
  }
};

#define PHASE(h, ph, expr)     \
  do {                         \
    PhaseScope ps_((h), (ph)); \
    CK(expr);                  \
  } while (0)

// After the stream was synchronised: add the recorded phase times.
static void collect_phases(hodlr_ctx *h) {
  if (!h->last_recs) return;
  for (auto &p : *h->last_recs) {
    float ms = 0.f;
    cudaError_t e = cudaEventElapsedTime(&ms, p.a, p.b);
    if (e == cudaSuccess) {
      h->phase_ms[p.phase] += ms;
      h->phase_n[p.phase] += 1;
    } else {
      if (debug_sync()) fprintf(stderr, "hodlr: phase %d timing: %s\n", p.phase, cudaGetErrorString(e));
      (void)cudaGetLastError();
    }
  }
  if (h->last_eager) destroy_recs(*h->last_recs);
  h->last_recs = nullptr;
}

static void free_ctx(hodlr_ctx *h) {
  if (!h) return;
  clear_graphs(h);
  destroy_recs(h->eager_recs);
  for (void *p : h->allocs) cudaFree(p);
  if (h->hst) cudaFreeHost(h->hst);
  for (auto &e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->pst) cudaStreamSynchronize(h->pst);
  for (auto &e : h->pready)
    if (e) cudaEventDestroy(e);
  if (h->pcopy) cudaEventDestroy(h->pcopy);
  if (h->pst) cudaStreamDestroy(h->pst);
  if (h->cst) cudaStreamDestroy(h->cst);
  for (auto &e : h->vready)
    if (e) cudaEventDestroy(e);
  for (auto &e : h->vcopied)
    if (e) cudaEventDestroy(e);
  if (h->vfork) cudaEventDestroy(h->vfork);
  if (h->vcs) cudaStreamDestroy(h->vcs);
  if (h->own_stream && h->st) cudaStreamDestroy(h->st);
  delete h;
}

// ----------------------------------------------------------------- sizes
static void plan_sizes(hodlr_ctx *h) {
  const int L = h->L, r = h->r, k = h->kmax;
  const size_t nbmax = L > 0 ? (size_t)h->nb(L - 1) : 1;
  size_t tb = std::max(nbmax * r * std::max(k, r), (size_t)r * std::max(k, r));
  size_t et = nbmax / 2 * 2 * (size_t)r * r;
  size_t red = 0;
  for (int l = 0; l < L; ++l) {
    const int nb = h->nb(l);
    const long long rows = h->rows(l);
    const size_t ct = (size_t)(l + 1) * r;
    tb = std::max(tb, (size_t)nb * r * ct);
    et = std::max(et, (size_t)h->nodes(l) * 2 * r * (size_t)l * r);
    et = std::max(et, (size_t)h->nodes(l) * 2 * r * (size_t)k);
    red = std::max(red, reduce_workspace_doubles(rows, nb, r, (int)ct, 8));
    red = std::max(red, reduce_workspace_doubles(rows, nb, r, r, 8));
    // a solve may use any nrhs <= kmax, and the split-K plans are not
    // monotone in the column count: size for every count
    for (int c = 1; c <= k; ++c) {
      red = std::max(red, reduce_workspace_doubles(rows, nb, r, c, 8));
      red = std::max(red, dw_reduce_workspace_doubles(rows, nb, r, c));
      if (rows % kOzChunk == 0) red = std::max(red, oz_reduce_workspace_doubles(rows, nb, r, c));
    }
  }
  h->tbuf_elems = tb;
  h->eta_elems = et;
  h->red_elems = red;
}

// ---------------------------------------------------------------- status
static int sync_status(hodlr_ctx *h, hodlr_solve_info *info) {
  CK(cudaMemcpyAsync(h->hst, h->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  DevStatus s = *h->hst;
  if (info) {
    info->iterations = s.iters;
    info->status = s.code;
    info->bad_index = s.index;
    info->rel_residual = s.resid;
  }
  if (s.code != HODLR_OK) {
    static const char *names[] = {"ok", "invalid argument", "cuda error", "singular leaf block",
                                  "singular capacitance system", "refinement did not converge",
                                  "non-finite input", "device wait timed out", "not factored",
                                  "out of memory"};
    char buf[160];
    snprintf(buf, sizeof buf, "%s (index %lld)", (s.code >= 0 && s.code <= 9) ? names[s.code] : "error",
             s.index);
    return set_err(s.code, buf);
  }
  return HODLR_OK;
}

// The handle's stream waits for the set-time preparation still running on the
// side stream (every call that reads the prepared copies, or writes the
// inputs by another route, comes through here first).
static int join_prep(hodlr_ctx *h) {
  if (h->plast) {
    CK(cudaStreamWaitEvent(h->st, h->plast, 0));
    h->plast = nullptr;
  }
  return HODLR_OK;
}

static int reset_status(hodlr_ctx *h) {
  CKS(join_prep(h));
  CK(cudaMemsetAsync(h->dst, 0, sizeof(DevStatus), h->st));
  return HODLR_OK;
}

// Run fn eagerly, or (after the first eager run of the same key) as a CUDA
// graph captured from fn.
template <typename F>
static int run_graphed(hodlr_ctx *h, GraphEntry &g, int &runs, F fn) {
  if (!h->use_graphs || runs == 0 || h->st == nullptr) {
    ++runs;
    destroy_recs(h->eager_recs);
    h->recs = &h->eager_recs;
    h->last_recs = &h->eager_recs;
    h->last_eager = true;
    int rc = fn();
    h->recs = nullptr;
    return rc;
  }
  if (!g.exec) {
    long long before = g_launches.load();
    destroy_recs(g.recs);
    h->recs = &g.recs;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    int rc = fn();
    h->recs = nullptr;
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(h->st, &graph);
    if (rc != HODLR_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    CK(ce);
    cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ie);
    g.kernels = g_launches.load() - before;
    g_launches.fetch_sub(g.kernels);  // counted on each replay instead
  }
  g_launches.fetch_add(g.kernels);
  h->last_recs = &g.recs;
  h->last_eager = false;
  CK(cudaGraphLaunch(g.exec, h->st));
  ++runs;
  return HODLR_OK;
}

// ----------------------------------------------------------- the sweeps
template <typename T> static T *LUptr(hodlr_ctx *h);
template <> double *LUptr<double>(hodlr_ctx *h) { return h->LU; }
template <> float *LUptr<float>(hodlr_ctx *h) { return h->LU32; }
template <typename T> static T *Utptr(hodlr_ctx *h);
template <> double *Utptr<double>(hodlr_ctx *h) { return h->Ut; }
template <> float *Utptr<float>(hodlr_ctx *h) { return h->Ut32; }
template <typename T> static const T *Vptr(hodlr_ctx *h);
template <> const double *Vptr<double>(hodlr_ctx *h) { return h->V; }
template <> const float *Vptr<float>(hodlr_ctx *h) { return h->V32; }

template <typename T> static T *Dinvptr(hodlr_ctx *h);
template <> double *Dinvptr<double>(hodlr_ctx *h) { return h->Dinv; }
template <> float *Dinvptr<float>(hodlr_ctx *h) { return h->Dinv32; }

// X := D^{-1} X (or D^{-T} X) on every leaf's rows: explicit inverse GEMM when
// the leaf size has a tuned kernel, LU triangular solves otherwise.
template <typename T>
static int leaf_solve(hodlr_ctx *h, T *X, long long ldx, int ncols, bool trans, const int *skip) {
  T *Dinv = Dinvptr<T>(h);
  if (Dinv)
    PHASE(h, HODLR_PHASE_LEAF_SOLVE,
          launch_leaf_apply<T>(Dinv, h->m, h->nleaf, X, ldx, ncols, trans, skip, h->st));
  else
    PHASE(h, HODLR_PHASE_LEAF_SOLVE,
          launch_leaf_getrs<T>(LUptr<T>(h), h->ipiv, h->m, h->nleaf, X, ldx, ncols, trans, skip, h->st));
  return HODLR_OK;
}

// eta = op(Sinv) RHS for the nodes of depth l (RHS from the T blocks).
static int cap_apply(hodlr_ctx *h, int l, int C, long long tb_stride, bool trans, const int *skip) {
  CapApplyArgs ca{};
  ca.Tb = h->Tbuf;
  ca.tb_stride = tb_stride;
  ca.scale = h->slev(l);
  ca.sinv = h->Sinv;
  ca.sinv2 = nullptr;
  ca.sinv32 = h->mixed ? h->Sinv32 : nullptr;
  ca.eta = h->eta;
  if (h->mixed) {  // FP32 T blocks in, FP32 eta out for the FP32 updates (the solve's row scaling applied)
    ca.Tb32 = h->Tbuf32;
    ca.eta32 = h->eta32;
    ca.out_scale = trans ? h->slev(l) : nullptr;
  }
  ca.r = h->r;
  ca.C = C;
  ca.nnode = h->nodes(l);
  ca.node_base = h->node_base(l);
  ca.trans = trans;
  ca.skip = skip;
  PHASE(h, HODLR_PHASE_CAPACITANCE, launch_cap_apply(ca, h->st));
  return HODLR_OK;
}

// The mixed path at leaf 128 factors its leaves by the blocked Gauss-Jordan
// kernel, which forms the explicit inverses only.
static bool leaf_inverse_only(const hodlr_ctx *h) { return h->mixed && h->m == 128 && h->Dinv32; }

static cudaError_t launch_mixed_leaf_factor(hodlr_ctx *h, DevStatus *st, cudaStream_t s) {
  const int m = h->m;
  const long long mm = (long long)m * m;
  if (leaf_inverse_only(h)) return launch_leaf_gj_inverse_f32(h->D, m, mm, m, h->nleaf, st, h->Dinv32, s);
  float *Dinv = h->Dinv32;
  const bool fused = Dinv && leaf_getrf_fused_inverse(m, sizeof(float));
  cudaError_t e = launch_leaf_getrf<float>(h->D, m, mm, h->LU32, h->ipiv, m, h->nleaf, st, fused ? Dinv : nullptr, s);
  if (e == cudaSuccess && Dinv && !fused) e = launch_leaf_inverse<float>(h->LU32, h->ipiv, m, h->nleaf, Dinv, s);
  return e;
}

// The leaf LU factors and pivots of a factored mixed handle whose
// factorisation formed only the inverses: formed now, from the leaf blocks.
static int ensure_leaf_lu(hodlr_ctx *h) {
  if (!h->lu_stale) return HODLR_OK;
  CKS(reset_status(h));
  CK(launch_leaf_getrf<float>(h->D, h->m, (long long)h->m * h->m, h->LU32, h->ipiv, h->m, h->nleaf, h->dst, nullptr,
                              h->st));
  CKS(sync_status(h, nullptr));
  h->lu_stale = false;
  return HODLR_OK;
}

// Factorisation sweep: leaf LU (+ explicit leaf inverses), Ut = D^{-1} U
// (all levels at once), then for depth L-1 .. 0: T = V^T [Ut_d | Ut_u],
// capacitance LU + inverse, eta = Sinv [s.T1d; s.T0d], Ut_d -= Ut_u eta.
static int prepare_level_v(hodlr_ctx *h, int l, long long row0, long long count, cudaStream_t ps);

template <typename T> static int factor_sweep(hodlr_ctx *h, bool leaves_done = false, bool streamed_v = false) {
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r;
  cudaStream_t s = h->st;
  if (streamed_v) {
    // the V copies of the levels that wait for them, deepest first and back
    // to back on their own stream (so that the host link never waits for the
    // SMs); each level's derived copies on the side stream after its copy;
    // both forked from the sweep and joined back into it level by level
    CK(cudaEventRecord(h->vfork, s));
    CK(cudaStreamWaitEvent(h->vcs, h->vfork, 0));
    CK(cudaStreamWaitEvent(h->pst, h->vfork, 0));
    for (int l = L - 1; l >= 0; --l) {
      if (h->vsrc[l]) {
        CK(cudaMemcpy2DAsync(h->Vlev(l), sizeof(double) * n, h->vsrc[l], sizeof(double) * h->vsrc_ld[l],
                             sizeof(double) * n, r, cudaMemcpyHostToDevice, h->vcs));
        CK(cudaEventRecord(h->vcopied[l], h->vcs));
        CK(cudaStreamWaitEvent(h->pst, h->vcopied[l], 0));
        CKS(prepare_level_v(h, l, 0, -1, h->pst));
      }
      CK(cudaEventRecord(h->vready[l], h->pst));
    }
    if (!h->vsrc[0]) {  // join the copy stream through the side stream's last event
      CK(cudaEventRecord(h->vcopied[0], h->vcs));
      CK(cudaStreamWaitEvent(h->pst, h->vcopied[0], 0));
      CK(cudaEventRecord(h->vready[0], h->pst));
    }
  }
  T *LU = LUptr<T>(h);
  T *Ut = Utptr<T>(h);
  const T *Vt = Vptr<T>(h);
  T *Dinv = Dinvptr<T>(h);
  const bool fused = Dinv && leaf_getrf_fused_inverse(m, sizeof(T));
  if (!leaves_done) {
    if (sizeof(T) == 4) {
      PHASE(h, HODLR_PHASE_LEAF_LU, launch_mixed_leaf_factor(h, h->dst, s));
    } else {
      PHASE(h, HODLR_PHASE_LEAF_LU,
            launch_leaf_getrf<T>(h->D, m, (long long)m * m, LU, h->ipiv, m, h->nleaf, h->dst, fused ? Dinv : nullptr,
                                 s));
      if (Dinv && !fused) PHASE(h, HODLR_PHASE_LEAF_LU, launch_leaf_inverse<T>(LU, h->ipiv, m, h->nleaf, Dinv, s));
    }
  }
  if (L == 0) return HODLR_OK;
  if (sizeof(T) == 4 && Dinv && m == 128) {
    // Utilde = D^{-1} U straight from the FP64 U (rounded as it is split or
    // staged): on the tensor cores, or the FMA tiles when the tuning asks
    PHASE(h, HODLR_PHASE_LEAF_SOLVE,
          launch_leaf_apply_f64src(reinterpret_cast<const float *>(Dinv), m, h->nleaf, h->U, n,
                                   reinterpret_cast<float *>(Ut), n, L * r, h->dst, s));
  } else {
    if (sizeof(T) == 8)
      CK(cudaMemcpyAsync(Ut, h->U, sizeof(double) * n * L * r, cudaMemcpyDeviceToDevice, s));
    else
      PHASE(h, HODLR_PHASE_MISC,
            (launch_convert<double, float>(h->U, n, reinterpret_cast<float *>(Ut), n, n, L * r, s)));
    CKS(leaf_solve<T>(h, Ut, n, L * r, false, nullptr));
  }
  for (int l = L - 1; l >= 0; --l) {
    const int nb = h->nb(l);
    const long long rows = h->rows(l);
    const int Cd = l * r, Ct = Cd + r;
    if (streamed_v) CK(cudaStreamWaitEvent(s, h->vready[l], 0));
    PHASE(h, HODLR_PHASE_REDUCE,
          launch_reduce_tn<T>(Vt + (long long)l * n * r, n, Ut, n, rows, nb, r, Ct, h->Tbuf, h->red, nullptr, s, h->dst,
                              sizeof(T) == 4 ? h->Tbuf32 : nullptr));
    CapFactorArgs cf{};
    cf.Tb = h->Tbuf;
    if (sizeof(T) == 4) cf.Tb32 = h->Tbuf32;
    cf.tb_stride = (long long)r * Ct;
    cf.scale = h->slev(l);
    cf.ucol = Cd;
    cf.cap_lu = h->capLU;
    cf.cap_ipiv = h->cap_ipiv;
    cf.sinv = h->Sinv;
    cf.sinv2 = nullptr;
    cf.sinv32 = h->mixed ? h->Sinv32 : nullptr;
    cf.r = r;
    cf.nnode = h->nodes(l);
    cf.node_base = h->node_base(l);
    cf.st = h->dst;
    PHASE(h, HODLR_PHASE_CAPACITANCE, launch_cap_factor(cf, s));
    if (Cd > 0) {
      CKS(cap_apply(h, l, Cd, (long long)r * Ct, false, nullptr));
      UpdateArgs ua{};
      ua.A = Ut + (long long)l * r * n;
      ua.lda = n;
      ua.a_bstride = rows;
      ua.B = h->eta;
      if (sizeof(T) == 4) ua.B32 = h->eta32;
      ua.ldb = 2 * r;
      ua.b_s1 = 2LL * r * Cd;
      ua.b_s2 = r;
      ua.C = Ut;
      ua.ldc = n;
      ua.c_bstride = rows;
      ua.M = (int)rows;
      ua.N = Cd;
      ua.K = r;
      ua.nbatch = nb;
      ua.alpha = -1.0;
      PHASE(h, HODLR_PHASE_UPDATE, launch_update_nn<T>(ua, s, h->dst));
    }
  }
  return HODLR_OK;
}

// X := A^{-1} X (or A^{-T} X) with the stored factors, X of type T (n x k, ldx).
template <typename T>
static int solve_sweep(hodlr_ctx *h, T *X, long long ldx, int k, bool trans, const int *skip) {
  const long long n = h->n;
  const int L = h->L, r = h->r;
  cudaStream_t s = h->st;
  T *Ut = Utptr<T>(h);
  const T *Vt = Vptr<T>(h);
  if (!trans) CKS(leaf_solve<T>(h, X, ldx, k, false, skip));
  for (int step = 0; step < L; ++step) {
    const int l = trans ? step : L - 1 - step;
    const int nb = h->nb(l);
    const long long rows = h->rows(l);
    const T *Ared = trans ? Ut + (long long)l * r * n : Vt + (long long)l * n * r;
    const T *Aupd = trans ? Vt + (long long)l * n * r : Ut + (long long)l * r * n;
    PHASE(h, HODLR_PHASE_REDUCE,
          launch_reduce_tn<T>(Ared, n, X, ldx, rows, nb, r, k, h->Tbuf, h->red, skip, s, h->dst,
                              sizeof(T) == 4 ? h->Tbuf32 : nullptr));
    CKS(cap_apply(h, l, k, (long long)r * k, trans, skip));
    UpdateArgs ua{};
    ua.A = Aupd;
    ua.lda = n;
    ua.a_bstride = rows;
    ua.B = h->eta;
    ua.ldb = 2 * r;
    ua.b_s1 = 2LL * r * k;
    ua.b_s2 = r;
    ua.b_flip = trans ? 1 : 0;
    ua.scale = trans ? h->slev(l) : nullptr;
    if (sizeof(T) == 4) {  // FP32 eta, scaled by the capacitance kernel
      ua.B32 = h->eta32;
      ua.scale = nullptr;
    }
    ua.C = X;
    ua.ldc = ldx;
    ua.c_bstride = rows;
    ua.M = (int)rows;
    ua.N = k;
    ua.K = r;
    ua.nbatch = nb;
    ua.alpha = -1.0;
    ua.skip = skip;
    PHASE(h, HODLR_PHASE_UPDATE, launch_update_nn<T>(ua, s, h->dst));
  }
  if (trans) CKS(leaf_solve<T>(h, X, ldx, k, true, skip));
  return HODLR_OK;
}

// Y = beta*Y0 + alpha * op(A) X in native FP64 (Y0 == nullptr: Y starts at 0).
static int matvec_fp64(hodlr_ctx *h, bool trans, const double *X, long long ldx, const double *Y0,
                       long long ldy0, double *Y, long long ldy, int k, double alpha, const int *skip) {
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r;
  cudaStream_t s = h->st;
  if (Y0)
    CK(launch_axpy(Y0, ldy0, Y, ldy, n, k, 1.0, false, skip, s));
  else
    CK(cudaMemset2DAsync(Y, sizeof(double) * ldy, 0, sizeof(double) * n, k, s));
  UpdateArgs la{};
  la.A = h->D;
  la.lda = m;
  la.a_bstride = (long long)m * m;
  la.a_trans = trans ? 1 : 0;
  la.B = X;
  la.ldb = ldx;
  la.b_s1 = 2LL * m;
  la.b_s2 = m;
  la.C = Y;
  la.ldc = ldy;
  la.c_bstride = m;
  la.M = m;
  la.N = k;
  la.K = m;
  la.nbatch = h->nleaf;
  la.alpha = alpha;
  la.skip = skip;
  PHASE(h, HODLR_PHASE_RESID_LEAF, launch_update_nn<double>(la, s));
  for (int l = 0; l < L; ++l) {
    const int nb = h->nb(l);
    const long long rows = h->rows(l);
    const double *Ared = trans ? h->Ulev(l) : h->Vlev(l);
    const double *Aupd = trans ? h->Vlev(l) : h->Ulev(l);
    PHASE(h, HODLR_PHASE_RESID_REDUCE, launch_reduce_tn<double>(Ared, n, X, ldx, rows, nb, r, k, h->Tbuf, h->red, skip, s));
    UpdateArgs ua{};
    ua.A = Aupd;
    ua.lda = n;
    ua.a_bstride = rows;
    ua.B = h->Tbuf;
    ua.ldb = r;
    ua.b_s1 = 2LL * r * k;
    ua.b_s2 = (long long)r * k;
    ua.b_flip = 1;
    ua.scale = h->slev(l);
    ua.C = Y;
    ua.ldc = ldy;
    ua.c_bstride = rows;
    ua.M = (int)rows;
    ua.N = k;
    ua.K = r;
    ua.nbatch = nb;
    ua.alpha = alpha;
    ua.skip = skip;
    PHASE(h, HODLR_PHASE_RESID_UPDATE, launch_update_nn<double>(ua, s));
  }
  return HODLR_OK;
}

// R = B - op(A) X with double-word (FP32 pair) arithmetic on the FP32 pipes.
static int residual_emulated(hodlr_ctx *h, bool trans, const double *X, long long ldx, const double *B,
                             long long ldb, double *R, long long ldr, int k, const int *skip) {
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r;
  cudaStream_t s = h->st;
  PHASE(h, HODLR_PHASE_MISC, launch_split(X, ldx, h->X2, n, n, k, skip, s));
  DwUpdateArgs la{};
  la.A = h->D2;
  la.lda = m;
  la.a_bstride = (long long)m * m;
  la.a_trans = trans ? 1 : 0;
  la.B = h->X2;
  la.ldb = n;
  la.b_s1 = 2LL * m;
  la.b_s2 = m;
  la.C = h->R2;
  la.ldc = n;
  la.c_bstride = m;
  la.Cinit = B;
  la.ldci = ldb;
  la.M = m;
  la.N = k;
  la.K = m;
  la.nbatch = h->nleaf;
  la.skip = skip;
  PHASE(h, HODLR_PHASE_RESID_LEAF, launch_dw_update(la, s));
  for (int l = 0; l < L; ++l) {
    const int nb = h->nb(l);
    const long long rows = h->rows(l);
    const float2 *U2l = h->U2 + (long long)l * n * r, *V2l = h->V2 + (long long)l * n * r;
    PHASE(h, HODLR_PHASE_RESID_REDUCE,
          launch_dw_reduce(trans ? U2l : V2l, n, h->X2, n, rows, nb, r, k, h->Tbuf, h->red, skip, s));
    PHASE(h, HODLR_PHASE_MISC, launch_scale_split(h->Tbuf, h->slev(l), r, (long long)nb * r * k, h->T2, skip, s));
    DwUpdateArgs ua{};
    ua.A = trans ? V2l : U2l;
    ua.lda = n;
    ua.a_bstride = rows;
    ua.B = h->T2;
    ua.ldb = r;
    ua.b_s1 = 2LL * r * k;
    ua.b_s2 = (long long)r * k;
    ua.b_flip = 1;
    ua.C = h->R2;
    ua.ldc = n;
    ua.c_bstride = rows;
    ua.M = (int)rows;
    ua.N = k;
    ua.K = r;
    ua.nbatch = nb;
    ua.skip = skip;
    PHASE(h, HODLR_PHASE_RESID_UPDATE, launch_dw_update(ua, s));
  }
  if (R) PHASE(h, HODLR_PHASE_MISC, launch_merge(h->R2, n, R, ldr, n, k, skip, s));
  return HODLR_OK;
}

// R = B - A X with the digit-product GEMMs on the tensor cores (forward only).
// With corr, the iterate is first updated in place: X := (first ? 0 : X) +
// corr (the FP32 correction), fused with its slicing.  With R == nullptr the
// result stays in the double-word buffer R2.
static int residual_tensor(hodlr_ctx *h, double *X, long long ldx, const double *B, long long ldb, double *R,
                           long long ldr, int k, const int *skip, const float *corr = nullptr,
                           bool first = false) {
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r;
  cudaStream_t s = h->st;
  if (corr)
    PHASE(h, HODLR_PHASE_MISC,
          launch_oz_slice_cols(first ? nullptr : X, ldx, n, k, h->Xsl, n, n * k, h->Xexp, skip, s, corr, X));
  else
    PHASE(h, HODLR_PHASE_MISC, launch_oz_slice_cols(X, ldx, n, k, h->Xsl, n, n * k, h->Xexp, skip, s));
  if (h->oz_tc) {
    // every level's reduction and T' digits first, then the leaf and all
    // update products in one pass
    PHASE(h, HODLR_PHASE_RESID_REDUCE,
          launch_oz_tc_reduce(h->Vsl, h->Vexp, h->Xsl, h->Xexp, n, L, r, k, h->lev_nb.data(), h->lev_rows.data(),
                              h->Tall, h->Tpart, skip, h->dst, s));
    const double *scales[kOzMaxLevels];
    for (int l = 0; l < L; ++l) scales[l] = h->slev(l);
    PHASE(h, HODLR_PHASE_MISC,
          launch_oz_slice_tprime_all(h->Tall, r, k, L, h->lev_nb.data(), scales, h->Tsl, h->Texp, skip, s));
    PHASE(h, HODLR_PHASE_RESID_UPDATE,
          launch_oz_tc_resid(h->Dsl, h->Dexp, h->Xsl, h->Xexp, h->Usl, h->Uexp, h->Tsl, h->Texp, n, m, L, r, k,
                             h->lev_nb.data(), h->lev_rows.data(), B, ldb, h->R2, n, skip, h->dst, s));
    if (R) PHASE(h, HODLR_PHASE_MISC, launch_merge(h->R2, n, R, ldr, n, k, skip, s));
    return HODLR_OK;
  }
  PHASE(h, HODLR_PHASE_RESID_LEAF,
        launch_oz_leaf(h->Dsl, h->Dexp, m, h->nleaf, h->Xsl, h->Xexp, n, k, B, ldb, h->R2, n, skip, s));
  for (int l = 0; l < L; ++l) {
    const int nb = h->nb(l);
    const long long rows = h->rows(l);
    PHASE(h, HODLR_PHASE_RESID_REDUCE,
          launch_oz_reduce(h->Vsl + (long long)l * r * n, (long long)L * r * n,
                           h->Vexp + (long long)l * (n / kOzChunk) * r, r, h->Xsl, h->Xexp, n, k, rows, nb, h->Tbuf,
                           h->red, skip, s));
    PHASE(h, HODLR_PHASE_MISC, launch_oz_slice_tprime(h->Tbuf, h->slev(l), r, k, nb, h->Tsl, h->Texp, skip, s));
    PHASE(h, HODLR_PHASE_RESID_UPDATE,
          launch_oz_update(h->Usl + (long long)l * n * r, (long long)L * n * r, h->Uexp + (long long)l * n, r,
                           h->Tsl, h->Texp, k, rows, nb, h->R2, n, skip, s));
  }
  if (R) PHASE(h, HODLR_PHASE_MISC, launch_merge(h->R2, n, R, ldr, n, k, skip, s));
  return HODLR_OK;
}

// R = B - op(A) X, FP64-accurate, with the handle's residual arithmetic.
static int residual(hodlr_ctx *h, bool trans, const double *X, long long ldx, const double *B, long long ldb,
                    double *R, long long ldr, int k, const int *skip) {
  if (h->oz && !trans) return residual_tensor(h, const_cast<double *>(X), ldx, B, ldb, R, ldr, k, skip);
  if (h->emulated) return residual_emulated(h, trans, X, ldx, B, ldb, R, ldr, k, skip);
  return matvec_fp64(h, trans, X, ldx, B, ldb, R, ldr, k, -1.0, skip);
}

// While the handle's stream is being captured (and no per-phase event nodes
// are recorded, which conditional bodies cannot hold): a graph conditional
// node of type WHILE whose body, captured from body() on the handle's body
// stream, runs again as long as a kernel of it (or one before the node) sets
// the condition.  Returns false in *used when the stream is not capturing.
static bool capturing_plain(hodlr_ctx *h) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->st, &cs) != cudaSuccess) return false;
  return cs == cudaStreamCaptureStatusActive && !h->profile;
}

static int cond_create(hodlr_ctx *h, cudaGraphConditionalHandle *hc) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  CK(cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
  CK(cudaGraphConditionalHandleCreate(hc, g, 0, cudaGraphCondAssignDefault));
  return HODLR_OK;
}

template <typename F>
static int cond_while(hodlr_ctx *h, cudaGraphConditionalHandle hc, F body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = hc;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
  CK(cudaStreamUpdateCaptureDependencies(h->st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  if (!h->cst) CK(cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking));
  cudaGraph_t bg = p.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(h->cst, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  cudaStream_t main = h->st;
  h->st = h->cst;
  const int rc = body();
  h->st = main;
  cudaGraph_t out = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(h->cst, &out);
  CKS(rc);
  CK(ce);
  return HODLR_OK;
}

// Mixed-precision solve with FP64 iterative refinement.  B (FP64, n x k) is
// overwritten by X.  All control stays on the device.  Run eagerly, the loop
// is unrolled to its maximum length and the refinement check sets st->done,
// which predicates every later kernel.  Captured into a graph, the first
// residual and check run once and the corrections are the body of a WHILE
// conditional node, repeated only while the check asks for another one.
static int mixed_solve(hodlr_ctx *h, double *B, long long ldb, int k, bool trans) {
  const long long n = h->n;
  const int *done = &h->dst->done;
  double *bn = h->norms, *rn = h->norms + (size_t)h->kmax * h->nsys;
  const int maxit = std::max(0, h->d.refine_max_iter);
  const bool cond = capturing_plain(h) && maxit > 0;
  cudaGraphConditionalHandle hc = 0;
  if (cond) CKS(cond_create(h, &hc));
  // the double-word residuals land in R2, and their norms and the next
  // right-hand side come from one fused pass; the tensor-core residual also
  // folds the correction into the slicing of the iterate
  const bool fused = h->emulated || (h->oz && !trans);
  const bool tensor = h->oz && !trans;
  const int P = h->forest ? h->nleaf : 64;
  const int *seg = h->forest ? h->seg_leaf : nullptr;
  auto norms = [&](const double *X, double *out, const int *skip) {
    if (!h->forest) return launch_colnorms(X, n, n, k, out, h->nwork, skip, h->st);
    return launch_seg_colnorms(X, n, h->m, h->nleaf, k, h->seg_leaf, h->nsys, out, h->nwork, skip, h->st);
  };
  // residual of the current iterate, its norms (and, fused, the next right-hand side)
  auto resid_step = [&](bool first) -> int {
    if (fused) {
      if (tensor)
        CKS(residual_tensor(h, h->X64, n, h->B64, n, nullptr, n, k, done, h->X32, first));
      else
        CKS(residual(h, trans, h->X64, n, h->B64, n, nullptr, n, k, done));
      PHASE(h, HODLR_PHASE_MISC, launch_resid_finish(h->R2, n, k, P, h->X32, h->nwork, done, h->st));
      PHASE(h, HODLR_PHASE_MISC, launch_partial_norms(h->nwork, P, k, seg, h->nsys, rn, done, h->st));
    } else {
      CKS(residual(h, trans, h->X64, n, h->B64, n, h->R64, n, k, done));
      CK(norms(h->R64, rn, done));
    }
    return HODLR_OK;
  };
  // a correction: the FP32 sweep on the residual, added to the iterate
  auto correction = [&]() -> int {
    if (!fused) CK((launch_convert<double, float>(h->R64, n, h->X32, n, n, k, h->st)));
    CKS(solve_sweep<float>(h, h->X32, n, k, trans, done));
    if (!tensor)
      PHASE(h, HODLR_PHASE_MISC,
            (launch_add_correction<float>(h->X64, n, h->X32, n, h->X64, n, n, k, done, h->st)));
    return HODLR_OK;
  };
  auto check = [&](int it) -> int {
    if (cond) CK(launch_refine_check_cond(rn, bn, k * h->nsys, h->d.refine_tol, h->dst, maxit, hc, h->st));
    else CK(launch_refine_check(rn, bn, k * h->nsys, h->d.refine_tol, h->dst, it < maxit ? 1 : 0, h->st));
    return HODLR_OK;
  };
  if (fused) {
    PHASE(h, HODLR_PHASE_MISC, launch_rhs_prepare(B, ldb, n, k, P, h->B64, h->X32, h->nwork, h->st));
    PHASE(h, HODLR_PHASE_MISC, launch_partial_norms(h->nwork, P, k, seg, h->nsys, bn, nullptr, h->st));
    CKS(solve_sweep<float>(h, h->X32, n, k, trans, nullptr));
    if (!tensor) PHASE(h, HODLR_PHASE_MISC, (launch_convert<float, double>(h->X32, n, h->X64, n, n, k, h->st)));
  } else {  // native FP64 residual
    CK(launch_axpy(B, ldb, h->B64, n, n, k, 1.0, false, nullptr, h->st));
    CK(norms(h->B64, bn, nullptr));
    CK((launch_convert<double, float>(h->B64, n, h->X32, n, n, k, h->st)));
    CKS(solve_sweep<float>(h, h->X32, n, k, trans, nullptr));
    CK((launch_convert<float, double>(h->X32, n, h->X64, n, n, k, h->st)));
  }
  CKS(resid_step(true));
  CKS(check(0));
  if (cond) {
    CKS(cond_while(h, hc, [&]() -> int {
      CKS(correction());
      CKS(resid_step(false));
      return check(1);
    }));
  } else {
    for (int it = 1; it <= maxit; ++it) {
      CKS(correction());
      CKS(resid_step(false));
      CKS(check(it));
    }
  }
  CK(launch_axpy(h->X64, n, B, ldb, n, k, 1.0, false, nullptr, h->st));
  return HODLR_OK;
}

// Input-derived copies of the mixed path, made when the inputs are set (so a
// factorisation only reads them): FP32 V for the sweeps and the double-word
// splits of D, U, V for the emulated residual.
static int prepare_leaves(hodlr_ctx *h, long long leaf0 = 0, long long count = -1, cudaStream_t ps = nullptr) {
  const cudaStream_t st = ps ? ps : h->st;
  if (count < 0) count = h->nleaf;
  if (h->emulated && count > 0) {
    const long long mm = (long long)h->m * h->m, dm = count * mm;
    if (h->oz)
      h->dw_stale = true;
    else
      CK(launch_split(h->D + leaf0 * mm, dm, h->D2 + leaf0 * mm, dm, dm, 1, nullptr, st));
  }
  if (h->oz && count > 0) {  // rows of the leaf blocks, each scaled by its own exponent
    const long long m = h->m, mm = m * m;
    CK(launch_oz_slice_rows(h->D + leaf0 * mm, m, mm, 1, m, count * m, (int)m, h->Dsl + leaf0 * mm, m,
                            h->n * m, h->Dexp + leaf0 * m, st));
  }
  return HODLR_OK;
}

// Level l, rows [row0, row0 + count) (default: all rows): the copies derived
// from U (prepare_level_u), from V (prepare_level_v), or both.
static int prepare_level_u(hodlr_ctx *h, int l, long long row0 = 0, long long count = -1,
                           cudaStream_t ps = nullptr) {
  if (!h->mixed) return HODLR_OK;
  const cudaStream_t st = ps ? ps : h->st;
  const long long n = h->n, off = (long long)l * n * h->r + row0;
  if (count < 0) count = n;
  if (h->emulated && h->oz) {
    h->dw_stale = true;
  } else if (h->emulated) {
    CK(launch_split(h->Ulev(l) + row0, n, h->U2 + off, n, count, h->r, nullptr, st));
  }
  if (h->oz) {  // U: row-scaled digits, rows of r contiguous entries
    const long long r = h->r, L = h->L;
    CK(launch_oz_slice_rows(h->Ulev(l) + row0, count, 0, 1, n, count, (int)r, h->Usl + l * n * r + row0 * r, r,
                            L * n * r, h->Uexp + l * n + row0, st));
  }
  return HODLR_OK;
}

static int prepare_level_v(hodlr_ctx *h, int l, long long row0 = 0, long long count = -1,
                           cudaStream_t ps = nullptr) {
  if (!h->mixed) return HODLR_OK;
  const cudaStream_t st = ps ? ps : h->st;
  const long long n = h->n, off = (long long)l * n * h->r + row0;
  if (count < 0) count = n;
  CK((launch_convert<double, float>(h->Vlev(l) + row0, n, h->V32 + off, n, count, h->r, st)));
  if (h->emulated && h->oz) {
    h->dw_stale = true;
  } else if (h->emulated) {
    CK(launch_split(h->Vlev(l) + row0, n, h->V2 + off, n, count, h->r, nullptr, st));
  }
  if (h->oz) {  // V: digits scaled per 64-row chunk of each column, column-major
    const long long r = h->r, L = h->L;
    CK(launch_oz_slice_cols(h->Vlev(l) + row0, n, count, (int)r, h->Vsl + l * r * n + row0, n, L * r * n,
                            h->Vexp + l * (n / kOzChunk) * r + (row0 / kOzChunk) * r, nullptr, st));
  }
  return HODLR_OK;
}

static int prepare_level(hodlr_ctx *h, int l, long long row0 = 0, long long count = -1, cudaStream_t ps = nullptr) {
  CKS(prepare_level_u(h, l, row0, count, ps));
  return prepare_level_v(h, l, row0, count, ps);
}

static bool any_streamed_v(const hodlr_ctx *h) {
  for (const double *p : h->vsrc)
    if (p) return true;
  return false;
}

// Copy the V of every level still waiting for a factorisation now, on the
// handle's stream (for calls that read V before one).
static int flush_streamed_v(hodlr_ctx *h) {
  for (int l = 0; l < h->L; ++l) {
    if (!h->vsrc[l]) continue;
    CKS(join_prep(h));
    CK(cudaMemcpy2DAsync(h->Vlev(l), sizeof(double) * h->n, h->vsrc[l], sizeof(double) * h->vsrc_ld[l],
                         sizeof(double) * h->n, h->r, cudaMemcpyHostToDevice, h->st));
    CKS(prepare_level_v(h, l, 0, -1, h->st));
    h->vsrc[l] = nullptr;
  }
  return HODLR_OK;
}

// The double-word copies of every leaf block and level (tensor-core mode),
// made when a transposed solve first needs them after the inputs changed.
// Rows a forest's shorter trees lack are zero in U and V, so whole-level
// splits equal the per-system ones.  Inside a caller's stream capture the
// copies are recorded into that graph and stay marked out of date.
static int ensure_dw_splits(hodlr_ctx *h) {
  if (!h->dw_stale) return HODLR_OK;
  const long long n = h->n, r = h->r, dm = (long long)h->nleaf * h->m * h->m;
  CK(launch_split(h->D, dm, h->D2, dm, dm, 1, nullptr, h->st));
  for (int l = 0; l < h->L; ++l) {
    CK(launch_split(h->Ulev(l), n, h->U2 + (long long)l * n * r, n, n, (int)r, nullptr, h->st));
    CK(launch_split(h->Vlev(l), n, h->V2 + (long long)l * n * r, n, n, (int)r, nullptr, h->st));
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(h->st, &cs));
  if (cs == cudaStreamCaptureStatusNone) h->dw_stale = false;
  return HODLR_OK;
}

// Set-time preparation of the copies derived from one input (input 0: the
// leaf blocks, 1 + l: level l) on a side stream, so that it overlaps the copy
// of the next input when the hodlr_set_* calls follow one another (from host
// memory the copies run at the host link's rate, the preparation on the SMs).
// Order: before the copy into an input, the handle's stream waits for that
// input's previous preparation (wait_prepared); the side stream waits for the
// copy; calls that read prepared copies join the side stream first
// (join_prep).  Inside a caller's stream capture it all stays on the
// handle's stream.
static bool side_prep_ok(hodlr_ctx *h) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return false;
  if (!h->pst) {
    if (cudaStreamCreateWithFlags(&h->pst, cudaStreamNonBlocking) != cudaSuccess) {
      h->pst = nullptr;
      return false;
    }
    if (cudaEventCreateWithFlags(&h->pcopy, cudaEventDisableTiming) != cudaSuccess) {
      h->pcopy = nullptr;
      return false;
    }
    h->pready.assign(1 + h->L, nullptr);
    for (auto &e : h->pready)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        e = nullptr;
        return false;
      }
  }
  if (!h->pcopy) return false;
  for (cudaEvent_t e : h->pready)
    if (!e) return false;  // a failed event creation keeps the preparation on the handle's stream
  return true;
}

static int wait_prepared(hodlr_ctx *h, int input) {
  if (h->pst && !h->pready.empty() && h->pready[input]) CK(cudaStreamWaitEvent(h->st, h->pready[input], 0));
  return HODLR_OK;
}

template <typename F>
static int prepare_input(hodlr_ctx *h, int input, F prep) {
  if (!h->mixed || !side_prep_ok(h)) {
    CKS(join_prep(h));
    return prep(h->st);
  }
  CK(cudaEventRecord(h->pcopy, h->st));
  CK(cudaStreamWaitEvent(h->pst, h->pcopy, 0));
  CKS(prep(h->pst));
  CK(cudaEventRecord(h->pready[input], h->pst));
  h->plast = h->pready[input];
  return HODLR_OK;
}

// Level geometry of one tree or of a forest (sys_levels: the trees' depths
// in decreasing order, so that every tree starts on a row that is a multiple
// of its own size and no block of a level straddles two trees).
static void set_geometry(hodlr_ctx *h, const std::vector<int> &sys_levels) {
  const int L = h->L;
  h->lev_nb.assign(L, 0);
  h->lev_rows.assign(L, 0);
  h->lev_base.assign(L, 0);
  int base = 0;
  for (int l = 0; l < L; ++l) {
    const int t = L - 1 - l;  // height above the leaves
    const long long c = (long long)h->m << t;
    long long covered = 0;
    for (int Li : sys_levels)
      if (Li > t) covered += (long long)h->m << Li;
    h->lev_rows[l] = c;
    h->lev_nb[l] = (int)(covered / c);
    h->lev_base[l] = base;
    base += h->lev_nb[l] / 2;
  }
  h->nnode = base;
}

static int check_common(const hodlr_desc &d) {
  if (d.levels > 0 && (d.rank < 1 || d.rank > 64))
    return set_err(HODLR_ERR_INVALID_ARG, "rank must be in [1, 64]");
  if (d.levels > 0 && (d.n >> d.levels) < 1) return set_err(HODLR_ERR_INVALID_ARG, "leaf too small");
  if (d.nrhs_max < 1) return set_err(HODLR_ERR_INVALID_ARG, "nrhs_max must be >= 1");
  if (d.precision != HODLR_PREC_FP64 && d.precision != HODLR_PREC_MIXED)
    return set_err(HODLR_ERR_INVALID_ARG, "unknown precision mode");
  if (d.precision == HODLR_PREC_MIXED && !(d.refine_tol > 0.0))
    return set_err(HODLR_ERR_INVALID_ARG, "mixed mode needs refine_tol > 0");
  if (d.precision == HODLR_PREC_MIXED && (d.residual < HODLR_RESID_FP64 || d.residual > HODLR_RESID_FP64_TENSOR))
    return set_err(HODLR_ERR_INVALID_ARG, "unknown residual mode");
  if ((long long)d.leaf * d.leaf * 8 > (1LL << 31)) return set_err(HODLR_ERR_INVALID_ARG, "leaf too large");
  return HODLR_OK;
}

// Allocate a handle for one tree (sys_levels = {L}) or for a forest of
// trees with the same leaf size and rank (sys_levels sorted in decreasing
// order; d.n = sum of leaf * 2^L_i and d.levels = the largest L_i).
static int create_ctx(const hodlr_desc &d, const std::vector<int> &sys_levels, hodlr_ctx **out) {
  hodlr_ctx *h = new hodlr_ctx();
  h->d = d;
  h->n = d.n;
  h->m = d.leaf;
  h->L = d.levels;
  h->r = d.levels > 0 ? d.rank : std::max(1, d.rank);
  h->nleaf = (int)(d.n / d.leaf);
  h->kmax = d.nrhs_max;
  h->mixed = d.precision == HODLR_PREC_MIXED;
  h->has_level.assign(h->L, 0);
  h->vsrc.assign(h->L, nullptr);
  h->vsrc_ld.assign(h->L, 0);
  h->nsys = (int)sys_levels.size();
  h->forest = h->nsys > 1;
  set_geometry(h, sys_levels);
  if (d.stream) {
    h->st = (cudaStream_t)d.stream;
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete h;
      return set_err(HODLR_ERR_CUDA, cudaGetErrorString(e));
    }
    h->own_stream = true;
  }
  plan_sizes(h);
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r, k = h->kmax;
  cudaError_t e = cudaSuccess;
#define ALLOC(ptr, T, cnt)                                                    \
  do {                                                                        \
    ptr = h->alloc<T>((size_t)(cnt), e);                                      \
    if (e != cudaSuccess) {                                                   \
      free_ctx(h);                                                            \
      return set_err(HODLR_ERR_OUT_OF_MEMORY, std::string("cudaMalloc ") + #ptr); \
    }                                                                         \
  } while (0)
  ALLOC(h->D, double, (size_t)h->nleaf * m * m);
  ALLOC(h->U, double, (size_t)n * L * r);
  ALLOC(h->V, double, (size_t)n * L * r);
  ALLOC(h->s, double, (size_t)std::max(1, L) * r);
  ALLOC(h->ipiv, int, (size_t)n);
  ALLOC(h->capLU, double, (size_t)std::max(1, h->nnode) * 4 * r * r);
  ALLOC(h->cap_ipiv, int, (size_t)std::max(1, h->nnode) * 2 * r);
  if (!h->mixed) ALLOC(h->Sinv, double, (size_t)std::max(1, h->nnode) * 4 * r * r);
  if (h->mixed) ALLOC(h->Sinv32, float, (size_t)std::max(1, h->nnode) * 4 * r * r);
  if (leaf_apply_supported(m)) {
    if (h->mixed)
      ALLOC(h->Dinv32, float, (size_t)h->nleaf * m * m);
    else
      ALLOC(h->Dinv, double, (size_t)h->nleaf * m * m);
  }
  if (h->mixed) {
    ALLOC(h->LU32, float, (size_t)h->nleaf * m * m);
    ALLOC(h->V32, float, (size_t)n * L * r);
    ALLOC(h->Ut32, float, (size_t)n * L * r);
    ALLOC(h->X32, float, (size_t)n * k);
    ALLOC(h->X64, double, (size_t)n * k);
    ALLOC(h->R64, double, (size_t)n * k);
    ALLOC(h->B64, double, (size_t)n * k);
    if (d.residual == HODLR_RESID_FP64_TENSOR && L > 0 && oz_supported(m, r)) {
      h->oz = true;
      const size_t S = kOzSlices;
      const int nbmax = h->nb(L - 1);
      ALLOC(h->Dsl, __nv_bfloat16, S * n * m);
      ALLOC(h->Dexp, int, (size_t)n);
      ALLOC(h->Usl, __nv_bfloat16, S * n * L * r);
      ALLOC(h->Uexp, int, (size_t)n * L);
      ALLOC(h->Vsl, __nv_bfloat16, S * n * L * r);
      ALLOC(h->Vexp, int, (size_t)(n / kOzChunk) * L * r);
      ALLOC(h->Xsl, __nv_bfloat16, S * n * k);
      ALLOC(h->Xexp, int, (size_t)(n / kOzChunk) * k);
      const char *no_tc = getenv("HODLR_NO_TCGEN05");  // A/B switch for the mma.sync kernels
      h->oz_tc = oz_tc_supported(m, r, k) && L <= 32 && !(no_tc && no_tc[0] == '1');
      size_t nball = 0;
      for (int l = 0; l < L; ++l) nball += (size_t)h->nb(l);
      const size_t nbt = h->oz_tc ? nball : (size_t)nbmax;
      ALLOC(h->Tsl, __nv_bfloat16, S * nbt * k * r);
      ALLOC(h->Texp, int, nbt * k);
      if (h->oz_tc) {
        ALLOC(h->Tall, double, nball * k * r);
        const size_t np = oz_tc_reduce_partials(n, L, r, k, h->lev_nb.data(), h->lev_rows.data());
        if (np) ALLOC(h->Tpart, double, np);
      }
    }
    if (d.residual == HODLR_RESID_FP64_EMULATED || d.residual == HODLR_RESID_FP64_TENSOR) {
      h->emulated = true;  // also the transposed solves of the tensor-core mode
      ALLOC(h->D2, float2, (size_t)h->nleaf * m * m);
      ALLOC(h->U2, float2, (size_t)n * L * r);
      ALLOC(h->V2, float2, (size_t)n * L * r);
      ALLOC(h->X2, float2, (size_t)n * k);
      ALLOC(h->R2, float2, (size_t)n * k);
      ALLOC(h->T2, float2, h->tbuf_elems);
    }
  } else {
    ALLOC(h->LU, double, (size_t)h->nleaf * m * m);
    ALLOC(h->Ut, double, (size_t)n * L * r);
  }
  ALLOC(h->Tbuf, double, h->tbuf_elems);
  ALLOC(h->Wbuf, double, h->tbuf_elems);
  ALLOC(h->eta, double, h->eta_elems);
  if (h->mixed) {
    ALLOC(h->eta32, float, h->eta_elems);
    ALLOC(h->Tbuf32, float, h->tbuf_elems);
  }
  ALLOC(h->red, double, h->red_elems);
  ALLOC(h->norms, double, 2 * (size_t)k * h->nsys);
  ALLOC(h->nwork, double, (size_t)k * std::max(64, h->forest ? h->nleaf : 0));
  if (h->forest) {
    ALLOC(h->seg_leaf, int, (size_t)h->nsys + 1);
    ALLOC(h->sfold, double, (size_t)r);
  }
  ALLOC(h->dst, DevStatus, 1);
  ALLOC(h->dst_leaf, DevStatus, 1);
#undef ALLOC
  if (cudaMallocHost(&h->hst, sizeof(DevStatus)) != cudaSuccess) {
    free_ctx(h);
    return set_err(HODLR_ERR_OUT_OF_MEMORY, "cudaMallocHost");
  }
  for (auto &ev : h->ev)
    if (cudaEventCreate(&ev) != cudaSuccess) {
      free_ctx(h);
      return set_err(HODLR_ERR_CUDA, "cudaEventCreate");
    }
  if (L > 0) {
    cudaError_t fe = launch_fill(h->s, (long long)L * r, 1.0, h->st);
    if (fe != cudaSuccess) {
      free_ctx(h);
      return set_err(HODLR_ERR_CUDA, cudaGetErrorString(fe));
    }
  }
  if (h->forest) {
    // rows of a level that a shorter tree does not have stay zero in U, V
    // and their derived copies; per-system leaf offsets for the norms
    std::vector<int> seg(1, 0);
    for (int Li : sys_levels) seg.push_back(seg.back() + (1 << Li));
    const size_t nlr = (size_t)n * L * r;
    bool ok = cudaMemcpy(h->seg_leaf, seg.data(), sizeof(int) * seg.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMemsetAsync(h->U, 0, sizeof(double) * nlr, h->st) == cudaSuccess;
    ok = ok && cudaMemsetAsync(h->V, 0, sizeof(double) * nlr, h->st) == cudaSuccess;
    if (h->V32) ok = ok && cudaMemsetAsync(h->V32, 0, sizeof(float) * nlr, h->st) == cudaSuccess;
    if (h->U2) ok = ok && cudaMemsetAsync(h->U2, 0, sizeof(float2) * nlr, h->st) == cudaSuccess;
    if (h->V2) ok = ok && cudaMemsetAsync(h->V2, 0, sizeof(float2) * nlr, h->st) == cudaSuccess;
    if (h->oz) {
      ok = ok && cudaMemsetAsync(h->Usl, 0, sizeof(__nv_bfloat16) * kOzSlices * nlr, h->st) == cudaSuccess;
      ok = ok && cudaMemsetAsync(h->Vsl, 0, sizeof(__nv_bfloat16) * kOzSlices * nlr, h->st) == cudaSuccess;
      ok = ok && cudaMemsetAsync(h->Uexp, 0, sizeof(int) * n * L, h->st) == cudaSuccess;
      ok = ok && cudaMemsetAsync(h->Vexp, 0, sizeof(int) * (n / kOzChunk) * L * r, h->st) == cudaSuccess;
    }
    if (!ok) {
      free_ctx(h);
      return set_err(HODLR_ERR_CUDA, "forest initialisation");
    }
  }
  if (cudaMemsetAsync(h->dst, 0, sizeof(DevStatus), h->st) != cudaSuccess ||
      cudaStreamSynchronize(h->st) != cudaSuccess) {
    free_ctx(h);
    return set_err(HODLR_ERR_CUDA, "initialisation");
  }
  *out = h;
  return HODLR_OK;
}

// ----------------------------------------------------------------- C ABI
extern "C" {

const char *hodlr_last_error_string(void) { return g_err.c_str(); }

int64_t hodlr_kernel_launches(void) { return (int64_t)g_launches.load(); }

int hodlr_create(const hodlr_desc *desc, hodlr_handle *out) {
  if (!desc || !out) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  const hodlr_desc &d = *desc;
  if (d.leaf < 1 || d.levels < 0 || d.levels > 24 || d.n != ((int64_t)d.leaf << d.levels))
    return set_err(HODLR_ERR_INVALID_ARG, "need n = leaf * 2^levels, leaf >= 1, 0 <= levels <= 24");
  CKS(check_common(d));
  return create_ctx(d, std::vector<int>(1, d.levels), out);
}

int hodlr_destroy(hodlr_handle h) {
  if (!h) return HODLR_OK;
  if (h->pst) cudaStreamSynchronize(h->pst);
  cudaStreamSynchronize(h->st);
  free_ctx(h);
  return HODLR_OK;
}

int hodlr_set_stream(hodlr_handle h, void *stream) {
  if (!h) return set_err(HODLR_ERR_INVALID_ARG, "null handle");
  if (h->pst) CK(cudaStreamSynchronize(h->pst));
  h->plast = nullptr;
  CK(cudaStreamSynchronize(h->st));
  if (h->own_stream) cudaStreamDestroy(h->st);
  h->own_stream = false;
  if (stream) {
    h->st = (cudaStream_t)stream;
  } else {
    CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    h->own_stream = true;
  }
  return HODLR_OK;
}

int hodlr_set_leaf_blocks(hodlr_handle h, const double *D, int64_t ld, int64_t leaf_stride) {
  if (!h || !D) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  if (ld < h->m) return set_err(HODLR_ERR_INVALID_ARG, "ld < leaf size");
  const int m = h->m;
  const long long mm = (long long)m * m;
  CKS(wait_prepared(h, 0));
  if (ld == m && leaf_stride == mm) {
    CK(cudaMemcpyAsync(h->D, D, sizeof(double) * mm * h->nleaf, cudaMemcpyDefault, h->st));
  } else {
    // column j of every leaf in one strided copy (host or device source)
    for (int j = 0; j < m; ++j)
      CK(cudaMemcpy2DAsync(h->D + (long long)j * m, sizeof(double) * mm, D + (long long)j * ld,
                           sizeof(double) * leaf_stride, sizeof(double) * m, h->nleaf, cudaMemcpyDefault,
                           h->st));
  }
  h->has_D = true;
  h->factored = false;
  h->leaves_prefactored = false;
  return prepare_input(h, 0, [&](cudaStream_t ps) -> int {
    CKS(prepare_leaves(h, 0, -1, ps));
    if (h->mixed && ps != h->st) {
      // the leaf LU (+ inverses) depends on the leaf blocks alone: it runs on
      // the side stream while the low-rank inputs are still being copied
      CK(cudaMemsetAsync(h->dst_leaf, 0, sizeof(DevStatus), ps));
      CK(launch_mixed_leaf_factor(h, h->dst_leaf, ps));
      h->leaves_prefactored = true;
    }
    return HODLR_OK;
  });
}

int hodlr_set_lowrank(hodlr_handle h, int level, const double *U, int64_t ldu, const double *V, int64_t ldv,
                      const double *s) {
  if (!h || !U || !V) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  if (level < 0 || level >= h->L) return set_err(HODLR_ERR_INVALID_ARG, "level out of range");
  if (ldu < h->n || ldv < h->n) return set_err(HODLR_ERR_INVALID_ARG, "ld < n");
  CKS(wait_prepared(h, 1 + level));
  // HODLR_FLAG_STREAM_INPUTS and V in pinned host memory: V's copy waits for
  // the factorisation, which overlaps it with the levels below this one
  bool defer = false;
  if (h->d.flags & HODLR_FLAG_STREAM_INPUTS) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, V) == cudaSuccess && a.type == cudaMemoryTypeHost) defer = true;
    (void)cudaGetLastError();
  }
  // plain (2-D) copies: the sources may be device or host memory
  CK(cudaMemcpy2DAsync(h->Ulev(level), sizeof(double) * h->n, U, sizeof(double) * ldu, sizeof(double) * h->n,
                       h->r, cudaMemcpyDefault, h->st));
  if (!defer)
    CK(cudaMemcpy2DAsync(h->Vlev(level), sizeof(double) * h->n, V, sizeof(double) * ldv, sizeof(double) * h->n,
                         h->r, cudaMemcpyDefault, h->st));
  h->vsrc[level] = defer ? V : nullptr;
  h->vsrc_ld[level] = ldv;
  if (s)
    CK(cudaMemcpyAsync(h->slev(level), s, sizeof(double) * h->r, cudaMemcpyDefault, h->st));
  else
    CK(launch_fill(h->slev(level), h->r, 1.0, h->st));
  h->has_level[level] = 1;
  h->factored = false;
  if (defer)
    return prepare_input(h, 1 + level, [&](cudaStream_t ps) { return prepare_level_u(h, level, 0, -1, ps); });
  return prepare_input(h, 1 + level, [&](cudaStream_t ps) { return prepare_level(h, level, 0, -1, ps); });
}

int hodlr_factor(hodlr_handle h) {
  if (!h) return set_err(HODLR_ERR_INVALID_ARG, "null handle");
  TuningScope tscope(&h->tune);
  if (!h->has_D) return set_err(HODLR_ERR_NOT_FACTORED, "leaf blocks not set");
  for (int l = 0; l < h->L; ++l)
    if (!h->has_level[l]) return set_err(HODLR_ERR_NOT_FACTORED, "low-rank level not set");
  h->factored = false;
  CKS(reset_status(h));
  // leaf LU already run on the side stream since the leaf blocks were set:
  // its status becomes the factorisation's, and the sweep starts after it
  const bool nl = h->leaves_prefactored;
  h->leaves_prefactored = false;
  if (nl) CK(cudaMemcpyAsync(h->dst, h->dst_leaf, sizeof(DevStatus), cudaMemcpyDeviceToDevice, h->st));
  // V copies streamed in by this factorisation (HODLR_FLAG_STREAM_INPUTS): their
  // own graphs, captured again when the host sources change
  bool sv = any_streamed_v(h) && side_prep_ok(h);
  if (sv && h->vready.empty()) {
    h->vready.assign(h->L, nullptr);
    h->vcopied.assign(h->L, nullptr);
    for (auto *v : {&h->vready, &h->vcopied})
      for (auto &e : *v)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) sv = false;
    if (cudaEventCreateWithFlags(&h->vfork, cudaEventDisableTiming) != cudaSuccess) sv = false;
    if (cudaStreamCreateWithFlags(&h->vcs, cudaStreamNonBlocking) != cudaSuccess) {
      h->vcs = nullptr;
      sv = false;
    }
  }
  if (sv && (!h->vcs || !h->vfork)) sv = false;
  if (!sv) CKS(flush_streamed_v(h));
  if (sv && h->sv_captured != h->vsrc) {
    clear_sv_graphs(h);
    h->sv_captured = h->vsrc;
  }
  GraphEntry &g = sv ? (nl ? h->factor_sv_nl_graph : h->factor_sv_graph) : (nl ? h->factor_nl_graph : h->factor_graph);
  int &runs = sv ? (nl ? h->factor_sv_nl_runs : h->factor_sv_runs) : (nl ? h->factor_nl_runs : h->factor_runs);
  CK(cudaEventRecord(h->ev[0], h->st));
  int rc = run_graphed(h, g, runs, [&]() -> int {
    if (h->mixed) return factor_sweep<float>(h, nl, sv);
    return factor_sweep<double>(h, nl, sv);
  });
  CKS(rc);
  if (sv) std::fill(h->vsrc.begin(), h->vsrc.end(), nullptr);
  CK(cudaEventRecord(h->ev[1], h->st));
  int fst = sync_status(h, nullptr);
  collect_phases(h);
  CKS(fst);
  cudaEventElapsedTime(&h->factor_ms, h->ev[0], h->ev[1]);
  h->factored = true;
  h->lu_stale = leaf_inverse_only(h);
  return HODLR_OK;
}

static int solve_impl(hodlr_handle h, double *B, int64_t ldb, int nrhs, hodlr_solve_info *info, bool trans) {
  if (!h || !B) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  TuningScope tscope(&h->tune);
  if (!h->factored) return set_err(HODLR_ERR_NOT_FACTORED, "call hodlr_factor first");
  if (nrhs < 1 || nrhs > h->kmax) return set_err(HODLR_ERR_INVALID_ARG, "nrhs out of range");
  if (ldb < h->n) return set_err(HODLR_ERR_INVALID_ARG, "ldb < n");
  CKS(reset_status(h));
  if (trans && h->mixed) CKS(ensure_dw_splits(h));
  CK(cudaEventRecord(h->ev[2], h->st));
  auto key = std::make_tuple((const double *)B, (long long)ldb, nrhs, trans ? 1 : 0);
  if (h->solve_graphs.size() > 32 && !h->solve_graphs.count(key)) {  // bound the graph cache
    for (auto &g : h->solve_graphs)
      if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    h->solve_graphs.clear();
    h->solve_runs.clear();
  }
  int rc = run_graphed(h, h->solve_graphs[key], h->solve_runs[key], [&]() -> int {
    CK(launch_check_finite(B, ldb, h->n, nrhs, h->dst, h->st));
    if (h->mixed) return mixed_solve(h, B, ldb, nrhs, trans);
    return solve_sweep<double>(h, B, ldb, nrhs, trans, nullptr);
  });
  CKS(rc);
  CK(cudaEventRecord(h->ev[3], h->st));
  if (info) {
    info->iterations = 0;
    info->rel_residual = -1.0;
  }
  int st = sync_status(h, info);
  collect_phases(h);
  cudaEventElapsedTime(&h->solve_ms, h->ev[2], h->ev[3]);
  if (st != HODLR_OK) return st;
  if (h->mixed && !h->hst->done) {
    char buf[128];
    snprintf(buf, sizeof buf, "refinement stopped at relative residual %.3e after %d corrections",
             h->hst->resid, h->hst->iters);
    if (info) info->status = HODLR_ERR_NOT_CONVERGED;
    return set_err(HODLR_ERR_NOT_CONVERGED, buf);
  }
  if (!h->mixed && info) info->rel_residual = -1.0;
  return HODLR_OK;
}

int hodlr_solve(hodlr_handle h, double *B, int64_t ldb, int nrhs, hodlr_solve_info *info) {
  return solve_impl(h, B, ldb, nrhs, info, false);
}

int hodlr_solve_transpose(hodlr_handle h, double *B, int64_t ldb, int nrhs, hodlr_solve_info *info) {
  return solve_impl(h, B, ldb, nrhs, info, true);
}

int hodlr_matvec(hodlr_handle h, int transpose, const double *X, int64_t ldx, double *Y, int64_t ldy, int nrhs) {
  if (!h || !X || !Y) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  TuningScope tscope(&h->tune);
  if (nrhs < 1 || nrhs > h->kmax) return set_err(HODLR_ERR_INVALID_ARG, "nrhs out of range");
  if (ldx < h->n || ldy < h->n) return set_err(HODLR_ERR_INVALID_ARG, "ld < n");
  CKS(reset_status(h));
  CKS(flush_streamed_v(h));
  CKS(matvec_fp64(h, transpose != 0, X, ldx, nullptr, 0, Y, ldy, nrhs, 1.0, nullptr));
  return sync_status(h, nullptr);
}

int hodlr_adjoint(hodlr_handle h, const double *x, int64_t ldx, const double *g, int64_t ldg, int nrhs,
                  hodlr_grads *gr) {
  if (!h || !x || !g || !gr) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  TuningScope tscope(&h->tune);
  if (!h->factored) return set_err(HODLR_ERR_NOT_FACTORED, "call hodlr_factor first");
  if (nrhs < 1 || nrhs > h->kmax) return set_err(HODLR_ERR_INVALID_ARG, "nrhs out of range");
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r, k = nrhs;
  // lambda = A^{-T} g, held in the caller's db if given, else in a scratch buffer
  double *lam = gr->db;
  long long ldl = gr->ldb;
  double *scratch = nullptr;
  if (!lam) {
    CK(cudaMallocAsync(&scratch, sizeof(double) * n * k, h->st));
    lam = scratch;
    ldl = n;
  } else if (ldl < n) {
    return set_err(HODLR_ERR_INVALID_ARG, "grads->ldb < n");
  }
  CK(launch_axpy(g, ldg, lam, ldl, n, k, 1.0, false, nullptr, h->st));
  int rc = solve_impl(h, lam, ldl, k, nullptr, true);
  if (rc != HODLR_OK) {
    if (scratch) cudaFreeAsync(scratch, h->st);
    return rc;
  }
  cudaStream_t s = h->st;
  if (gr->dD) {
    CK(cudaMemsetAsync(gr->dD, 0, sizeof(double) * h->nleaf * m * m, s));
    UpdateArgs ua{};
    ua.A = lam;
    ua.lda = ldl;
    ua.a_bstride = m;
    ua.B = x;
    ua.ldb = ldx;
    ua.b_s1 = 2LL * m;
    ua.b_s2 = m;
    ua.b_trans = 1;
    ua.C = gr->dD;
    ua.ldc = m;
    ua.c_bstride = (long long)m * m;
    ua.M = m;
    ua.N = m;
    ua.K = k;
    ua.nbatch = h->nleaf;
    ua.alpha = -1.0;
    CK(launch_update_nn<double>(ua, s));
  }
  for (int l = 0; l < L && (gr->dU || gr->dV || gr->ds); ++l) {
    const int nb = h->nb(l);
    const long long rows = h->rows(l);
    CK(launch_reduce_tn<double>(h->Vlev(l), n, x, ldx, rows, nb, r, k, h->Tbuf, h->red, nullptr, s));
    CK(launch_reduce_tn<double>(h->Ulev(l), n, lam, ldl, rows, nb, r, k, h->Wbuf, h->red, nullptr, s));
    for (int which = 0; which < 2; ++which) {
      double *dst = which == 0 ? gr->dU : gr->dV;
      if (!dst) continue;
      dst += (long long)l * n * r;
      CK(cudaMemsetAsync(dst, 0, sizeof(double) * n * r, s));
      UpdateArgs ua{};
      ua.A = which == 0 ? lam : x;
      ua.lda = which == 0 ? ldl : ldx;
      ua.a_bstride = rows;
      ua.B = which == 0 ? h->Tbuf : h->Wbuf;
      ua.ldb = r;
      ua.b_s1 = 2LL * r * k;
      ua.b_s2 = (long long)r * k;
      ua.b_flip = 1;
      ua.b_trans = 1;
      ua.scale = h->slev(l);
      ua.scale_cols = 1;
      ua.C = dst;
      ua.ldc = n;
      ua.c_bstride = rows;
      ua.M = (int)rows;
      ua.N = r;
      ua.K = k;
      ua.nbatch = nb;
      ua.alpha = -1.0;
      CK(launch_update_nn<double>(ua, s));
    }
    if (gr->ds) CK(launch_scale_grad(h->Wbuf, h->Tbuf, r, k, nb, gr->ds + (long long)l * r, s));
  }
  if (scratch) CK(cudaFreeAsync(scratch, s));
  CKS(sync_status(h, nullptr));
  return HODLR_OK;
}

int hodlr_get_factors(hodlr_handle h, double *leaf_lu, int32_t *leaf_ipiv, double *utilde, double *cap_lu,
                      int32_t *cap_ipiv) {
  if (!h) return set_err(HODLR_ERR_INVALID_ARG, "null handle");
  if (!h->factored) return set_err(HODLR_ERR_NOT_FACTORED, "not factored");
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r;
  cudaStream_t s = h->st;
  if (leaf_lu || leaf_ipiv) CKS(ensure_leaf_lu(h));
  if (leaf_lu) {
    if (h->mixed)
      CK((launch_convert<float, double>(h->LU32, (long long)h->nleaf * m * m, leaf_lu, (long long)h->nleaf * m * m,
                                        (long long)h->nleaf * m * m, 1, s)));
    else
      CK(cudaMemcpyAsync(leaf_lu, h->LU, sizeof(double) * h->nleaf * m * m, cudaMemcpyDeviceToDevice, s));
  }
  if (leaf_ipiv) CK(cudaMemcpyAsync(leaf_ipiv, h->ipiv, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
  if (utilde && L > 0) {
    if (h->mixed)
      CK((launch_convert<float, double>(h->Ut32, n, utilde, n, n, L * r, s)));
    else
      CK(cudaMemcpyAsync(utilde, h->Ut, sizeof(double) * n * L * r, cudaMemcpyDeviceToDevice, s));
  }
  if (cap_lu && h->nnode > 0)
    CK(cudaMemcpyAsync(cap_lu, h->capLU, sizeof(double) * h->nnode * 4 * r * r, cudaMemcpyDeviceToDevice, s));
  if (cap_ipiv && h->nnode > 0)
    CK(cudaMemcpyAsync(cap_ipiv, h->cap_ipiv, sizeof(int) * h->nnode * 2 * r, cudaMemcpyDeviceToDevice, s));
  CK(cudaStreamSynchronize(s));
  return HODLR_OK;
}

int hodlr_get_inputs(hodlr_handle h, double *D, int64_t ld, int64_t leaf_stride, double *U, double *V,
                     double *s) {
  if (!h) return set_err(HODLR_ERR_INVALID_ARG, "null handle");
  CKS(flush_streamed_v(h));
  const int m = h->m;
  const long long mm = (long long)m * m, n = h->n;
  cudaStream_t st = h->st;
  if (D) {
    if (ld < m) return set_err(HODLR_ERR_INVALID_ARG, "ld < leaf size");
    for (int j = 0; j < m; ++j)
      CK(cudaMemcpy2DAsync(D + (long long)j * ld, sizeof(double) * leaf_stride, h->D + (long long)j * m,
                           sizeof(double) * mm, sizeof(double) * m, h->nleaf, cudaMemcpyDefault, st));
  }
  const size_t lvl = sizeof(double) * n * h->L * h->r;
  if (U && lvl) CK(cudaMemcpyAsync(U, h->U, lvl, cudaMemcpyDefault, st));
  if (V && lvl) CK(cudaMemcpyAsync(V, h->V, lvl, cudaMemcpyDefault, st));
  if (s && h->L) CK(cudaMemcpyAsync(s, h->s, sizeof(double) * h->L * h->r, cudaMemcpyDefault, st));
  CK(cudaStreamSynchronize(st));
  return HODLR_OK;
}

int hodlr_profile(hodlr_handle h, int enable, double *phase_ms, int64_t *phase_launches, int nphase) {
  if (!h) return set_err(HODLR_ERR_INVALID_ARG, "null handle");
  if (phase_ms || phase_launches) {
    for (int p = 0; p < nphase && p < HODLR_NUM_PHASES; ++p) {
      if (phase_ms) phase_ms[p] = h->phase_ms[p];
      if (phase_launches) phase_launches[p] = h->phase_n[p];
    }
    for (int p = 0; p < HODLR_NUM_PHASES; ++p) {
      h->phase_ms[p] = 0.0;
      h->phase_n[p] = 0;
    }
  }
  if (enable >= 0 && (enable != 0) != h->profile) {
    CK(cudaStreamSynchronize(h->st));
    clear_graphs(h);  // captured graphs carry (or lack) the timing events
    h->profile = enable != 0;
  }
  return HODLR_OK;
}

int hodlr_last_timings(hodlr_handle h, double *factor_ms, double *solve_ms) {
  if (!h) return set_err(HODLR_ERR_INVALID_ARG, "null handle");
  if (factor_ms) *factor_ms = h->factor_ms;
  if (solve_ms) *solve_ms = h->solve_ms;
  return HODLR_OK;
}

int hodlr_generate(hodlr_handle h, uint64_t seed, double shift, int orthonormal, double decay, double *B,
                   int64_t ldb, int nrhs) {
  if (!h) return set_err(HODLR_ERR_INVALID_ARG, "null handle");
  TuningScope tscope(&h->tune);
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r;
  cudaStream_t s = h->st;
  CKS(reset_status(h));
  std::fill(h->vsrc.begin(), h->vsrc.end(), nullptr);  // V is generated here
  CK(launch_gen_leaves(h->D, m, h->nleaf, seed, shift, s));
  h->has_D = true;
  h->leaves_prefactored = false;
  CKS(prepare_leaves(h));
  double *tmp = nullptr;
  if (orthonormal && L > 0) CK(cudaMallocAsync(&tmp, sizeof(double) * n * r, s));
  for (int l = 0; l < L; ++l) {
    const int nb = h->nb(l);
    const long long rows = h->rows(l);
    for (int w = 0; w < 2; ++w) {
      double *X = w == 0 ? h->Ulev(l) : h->Vlev(l);
      const unsigned long long stream = 0x100ull + 2ull * l + w;
      CK(launch_gaussian(X, n, n, r, seed, stream, orthonormal ? 1.0 : 1.0 / std::sqrt((double)rows), s));
      if (!orthonormal) continue;
      for (int pass = 0; pass < 2; ++pass) {  // CholeskyQR2 per child block
        CK(launch_reduce_tn<double>(X, n, X, n, rows, nb, r, r, h->Tbuf, h->red, nullptr, s));
        CK(launch_chol_inv(h->Tbuf, h->eta, r, nb, h->dst, s));
        CK(cudaMemsetAsync(tmp, 0, sizeof(double) * n * r, s));
        UpdateArgs ua{};
        ua.A = X;
        ua.lda = n;
        ua.a_bstride = rows;
        ua.B = h->eta;
        ua.ldb = r;
        ua.b_s1 = 2LL * r * r;
        ua.b_s2 = (long long)r * r;
        ua.C = tmp;
        ua.ldc = n;
        ua.c_bstride = rows;
        ua.M = (int)rows;
        ua.N = r;
        ua.K = r;
        ua.nbatch = nb;
        ua.alpha = 1.0;
        CK(launch_update_nn<double>(ua, s));
        CK(cudaMemcpyAsync(X, tmp, sizeof(double) * n * r, cudaMemcpyDeviceToDevice, s));
      }
    }
    std::vector<double> sv(r, 1.0);
    if (decay > 0)
      for (int i = 0; i < r; ++i) sv[i] = std::pow(10.0, -decay * i / r);
    CK(cudaMemcpyAsync(h->slev(l), sv.data(), sizeof(double) * r, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // sv is pageable host memory
    h->has_level[l] = 1;
    CKS(prepare_level(h, l));
  }
  if (tmp) CK(cudaFreeAsync(tmp, s));
  if (B) CK(launch_gaussian(B, ldb, n, nrhs, seed, 0xBull, 1.0, s));
  h->factored = false;
  return sync_status(h, nullptr);
}

// --------------------------------------------------- reference hsolve
static int is_device_ptr(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int hodlr_hsolve_ex(int nrow, int nrhs, int rank, int nPart, int LD, double *K, double *U, double *V,
                    int precision, void *stream, hodlr_solve_info *info) {
  if (!K || !U || nrow < 1 || nPart < 1 || nrhs < 1 || LD < nrow)
    return set_err(HODLR_ERR_INVALID_ARG, "hsolve: bad arguments");
  if ((nPart & (nPart - 1)) != 0 || nrow % nPart != 0)
    return set_err(HODLR_ERR_INVALID_ARG, "hsolve: nPart must be a power of two dividing nrow");
  int L = 0;
  while ((1 << L) < nPart) ++L;
  const int m = nrow / nPart;
  if (L > 0 && (!V || rank < 1 || rank > 64)) return set_err(HODLR_ERR_INVALID_ARG, "hsolve: rank in [1,64]");
  const int r = L > 0 ? rank : 1;
  const int ucols = nrhs + L * r;
  const bool dev = is_device_ptr(K) && is_device_ptr(U) && (L == 0 || is_device_ptr(V));
  if (stream && !dev) return set_err(HODLR_ERR_INVALID_ARG, "hsolve_ex: a stream needs device pointers");
  hodlr_desc d{};
  d.n = nrow;
  d.leaf = m;
  d.levels = L;
  d.rank = r;
  d.nrhs_max = nrhs;
  d.precision = precision;
  d.residual = HODLR_RESID_FP64_TENSOR;
  d.refine_tol = 1e-12;
  d.refine_max_iter = 10;
  d.stream = stream;
  hodlr_handle h = nullptr;
  CKS(hodlr_create(&d, &h));
  double *dK = K, *dU = U, *dV = V;
  long long ld = LD;
  int rc = HODLR_OK;
  std::vector<void *> tmp;
  auto fail = [&](int code) {
    for (void *p : tmp) cudaFree(p);
    hodlr_destroy(h);
    return code;
  };
  if (!dev) {  // stage host buffers through the device, packed (ld = nrow)
    ld = nrow;
    const size_t bk = sizeof(double) * nrow * m, bu = sizeof(double) * nrow * ucols,
                 bv = sizeof(double) * nrow * r;
    dK = dU = dV = nullptr;
    if (cudaMalloc(&dK, bk) == cudaSuccess) tmp.push_back(dK);
    if (cudaMalloc(&dU, bu) == cudaSuccess) tmp.push_back(dU);
    if (cudaMalloc(&dV, bv) == cudaSuccess) tmp.push_back(dV);
    if (tmp.size() != 3) return fail(set_err(HODLR_ERR_OUT_OF_MEMORY, "hsolve: staging buffers"));
    if (cudaMemcpy2DAsync(dK, sizeof(double) * nrow, K, sizeof(double) * LD, sizeof(double) * nrow, m,
                          cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
        cudaMemcpy2DAsync(dU, sizeof(double) * nrow, U, sizeof(double) * LD, sizeof(double) * nrow, ucols,
                          cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
        (L > 0 && cudaMemcpy2DAsync(dV, sizeof(double) * nrow, V, sizeof(double) * LD, sizeof(double) * nrow, r,
                                    cudaMemcpyHostToDevice, h->st) != cudaSuccess))
      return fail(set_err(HODLR_ERR_CUDA, "hsolve: host to device copy"));
  }
  if ((rc = hodlr_set_leaf_blocks(h, dK, ld, m)) != HODLR_OK) return fail(rc);
  for (int l = 0; l < L; ++l)
    if ((rc = hodlr_set_lowrank(h, l, dU + (long long)(nrhs + l * r) * ld, ld, dV, ld, nullptr)) != HODLR_OK)
      return fail(rc);
  if ((rc = hodlr_factor(h)) != HODLR_OK) return fail(rc);
  if ((rc = hodlr_solve(h, dU, ld, nrhs, info)) != HODLR_OK) return fail(rc);
  // write back: K <- leaf LU (stacked, ld), U columns nrhs.. <- Utilde
  cudaStream_t s = h->st;
  if ((rc = ensure_leaf_lu(h)) != HODLR_OK) return fail(rc);
  {
    cudaError_t e = h->mixed ? launch_unpack_leaves<float>(h->LU32, dK, ld, m, m, h->nleaf, s)
                             : launch_unpack_leaves<double>(h->LU, dK, ld, m, m, h->nleaf, s);
    if (e != cudaSuccess) return fail(set_err(HODLR_ERR_CUDA, "hsolve: LU write-back"));
  }
  if (L > 0) {
    cudaError_t e;
    if (h->mixed)
      e = launch_convert<float, double>(h->Ut32, h->n, dU + (long long)nrhs * ld, ld, h->n, L * r, s);
    else
      e = cudaMemcpy2DAsync(dU + (long long)nrhs * ld, sizeof(double) * ld, h->Ut, sizeof(double) * h->n,
                            sizeof(double) * h->n, L * r, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return fail(set_err(HODLR_ERR_CUDA, "hsolve: Utilde write-back"));
  }
  if (!dev) {
    if (cudaMemcpy2DAsync(K, sizeof(double) * LD, dK, sizeof(double) * nrow, sizeof(double) * nrow, m,
                          cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpy2DAsync(U, sizeof(double) * LD, dU, sizeof(double) * nrow, sizeof(double) * nrow, ucols,
                          cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return fail(set_err(HODLR_ERR_CUDA, "hsolve: device to host copy"));
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(set_err(HODLR_ERR_CUDA, "hsolve: sync"));
  return fail(HODLR_OK);
}

int hodlr_hsolve(int nrow, int nrhs, int rank, int nPart, int LD, double *K, double *U, double *V) {
  return hodlr_hsolve_ex(nrow, nrhs, rank, nPart, LD, K, U, V, HODLR_PREC_FP64, nullptr, nullptr);
}

// ------------------------------------------------- reference-structured init
// Device copies of the leaf sizes and their prefix offsets (rows, or block
// elements with squares) for the padding kernels.
static int irregular_tables(int nleaf, const int32_t *sz, int m_max, bool squares, int **dsz, long long **doff,
                            long long *total, cudaStream_t s) {
  if (nleaf < 1 || !sz || m_max < 1) return set_err(HODLR_ERR_INVALID_ARG, "bad leaf sizes");
  std::vector<int> h_sz(nleaf);
  std::vector<long long> h_off(nleaf);
  long long acc = 0;
  for (int i = 0; i < nleaf; ++i) {
    if (sz[i] < 1 || sz[i] > m_max) return set_err(HODLR_ERR_INVALID_ARG, "leaf size outside [1, m_max]");
    h_sz[i] = sz[i];
    h_off[i] = acc;
    acc += squares ? (long long)sz[i] * sz[i] : sz[i];
  }
  *total = acc;
  *dsz = nullptr;
  *doff = nullptr;
  CK(cudaMallocAsync((void **)dsz, sizeof(int) * nleaf, s));
  CK(cudaMallocAsync((void **)doff, sizeof(long long) * nleaf, s));
  CK(cudaMemcpyAsync(*dsz, h_sz.data(), sizeof(int) * nleaf, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(*doff, h_off.data(), sizeof(long long) * nleaf, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));  // the host vectors go out of scope
  return HODLR_OK;
}

static int pad_rows_impl(int nleaf, const int32_t *sz, int m_max, int cols, const double *src, int64_t lds,
                         double *dst, int64_t ldd, void *stream, bool unpad) {
  if (!src || !dst || cols < 0) return set_err(HODLR_ERR_INVALID_ARG, "bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  int *dsz = nullptr;
  long long *doff = nullptr, packed = 0;
  const int rc = irregular_tables(nleaf, sz, m_max, false, &dsz, &doff, &packed, s);
  if (rc != HODLR_OK) {
    if (dsz) cudaFreeAsync(dsz, s);
    if (doff) cudaFreeAsync(doff, s);
    return rc;
  }
  const long long padded = (long long)nleaf * m_max;
  cudaError_t e = cudaSuccess;
  if ((unpad ? lds < padded || ldd < packed : lds < packed || ldd < padded))
    e = cudaErrorInvalidValue;
  else
    e = launch_pad_rows(doff, dsz, nleaf, m_max, cols, src, lds, dst, ldd, unpad, s);
  cudaFreeAsync(dsz, s);
  cudaFreeAsync(doff, s);
  if (e == cudaErrorInvalidValue) return set_err(HODLR_ERR_INVALID_ARG, "leading dimension too small");
  CK(e);
  CK(cudaStreamSynchronize(s));
  return HODLR_OK;
}

int hodlr_pad_rows(int nleaf, const int32_t *sz, int m_max, int cols, const double *src, int64_t lds, double *dst,
                   int64_t ldd, void *stream) {
  return pad_rows_impl(nleaf, sz, m_max, cols, src, lds, dst, ldd, stream, false);
}

int hodlr_unpad_rows(int nleaf, const int32_t *sz, int m_max, int cols, const double *src, int64_t lds, double *dst,
                     int64_t ldd, void *stream) {
  return pad_rows_impl(nleaf, sz, m_max, cols, src, lds, dst, ldd, stream, true);
}

int hodlr_pad_leaf_blocks(int nleaf, const int32_t *sz, int m_max, const double *src, double *dst, void *stream) {
  if (!src || !dst) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  int *dsz = nullptr;
  long long *doff = nullptr, total = 0;
  const int rc = irregular_tables(nleaf, sz, m_max, true, &dsz, &doff, &total, s);
  if (rc != HODLR_OK) {
    if (dsz) cudaFreeAsync(dsz, s);
    if (doff) cudaFreeAsync(doff, s);
    return rc;
  }
  const cudaError_t e = launch_pad_leaf_blocks(doff, dsz, nleaf, m_max, src, dst, s);
  cudaFreeAsync(dsz, s);
  cudaFreeAsync(doff, s);
  CK(e);
  CK(cudaStreamSynchronize(s));
  return HODLR_OK;
}

int hodlr_draw_seeds(int64_t master, int n, int64_t *seeds) {
  if (n < 0 || (n > 0 && !seeds)) return set_err(HODLR_ERR_INVALID_ARG, "bad seed count or null output");
  unsigned long long x = lcg_seed(master);
  for (int i = 0; i < n; ++i) {
    x = lcg_step(x);
    seeds[i] = (int64_t)(x >> 17);  // lrand48: the top 31 bits of the state
  }
  return HODLR_OK;
}

// The per-partition seeds (host array) on the device, for the fill kernels.
static int seeds_to_device(const int64_t *seeds, int npart, long long **out, cudaStream_t s) {
  *out = nullptr;
  CK(cudaMallocAsync((void **)out, sizeof(long long) * std::max(1, npart), s));
  CK(cudaMemcpyAsync(*out, seeds, sizeof(long long) * npart, cudaMemcpyHostToDevice, s));
  return HODLR_OK;
}

int hodlr_rand_matrix(const int64_t *seeds, int npart, int64_t rows, int cols, double offset, double *A,
                      int64_t lda, void *stream) {
  if (!seeds || !A || npart < 1 || rows < 1 || cols < 0) return set_err(HODLR_ERR_INVALID_ARG, "bad argument");
  if (lda < (int64_t)npart * rows) return set_err(HODLR_ERR_INVALID_ARG, "lda < npart * rows");
  cudaStream_t s = (cudaStream_t)stream;
  long long *dseeds = nullptr;
  CKS(seeds_to_device(seeds, npart, &dseeds, s));
  cudaError_t e = launch_rand_block(dseeds, npart, rows, cols, offset, A, lda, s);
  cudaFreeAsync(dseeds, s);
  CK(e);
  CK(cudaStreamSynchronize(s));
  return HODLR_OK;
}

int hodlr_set_seeded(hodlr_handle h, const int64_t *useeds, const int64_t *vseeds, const int64_t *dseeds,
                     double offset) {
  if (!h || !useeds || !vseeds || !dseeds) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  CKS(join_prep(h));  // the inputs are rewritten: set-time preparation still reading them ends first
  if (h->forest) return set_err(HODLR_ERR_INVALID_ARG, "batch handles take hodlr_batch_set_* inputs");
  std::fill(h->vsrc.begin(), h->vsrc.end(), nullptr);
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r, nl = h->nleaf;
  cudaStream_t s = h->st;
  long long *su = nullptr, *sv = nullptr, *sd = nullptr;
  double *Dg = nullptr;
  int rc = seeds_to_device(useeds, nl, &su, s);
  if (rc == HODLR_OK) rc = seeds_to_device(vseeds, nl, &sv, s);
  if (rc == HODLR_OK) rc = seeds_to_device(dseeds, nl, &sd, s);
  if (rc == HODLR_OK && cudaMallocAsync((void **)&Dg, sizeof(double) * n, s) != cudaSuccess)
    rc = set_err(HODLR_ERR_OUT_OF_MEMORY, "cudaMallocAsync");
  // U, V: N x r, one m-row partition per leaf; D: N entries (+ offset).
  // Without levels (one dense block) the leaf block uses scratch U and V.
  double *Ub = nullptr, *Vb = nullptr;
  if (rc == HODLR_OK && L == 0 &&
      (cudaMallocAsync((void **)&Ub, sizeof(double) * n * r, s) != cudaSuccess ||
       cudaMallocAsync((void **)&Vb, sizeof(double) * n * r, s) != cudaSuccess))
    rc = set_err(HODLR_ERR_OUT_OF_MEMORY, "cudaMallocAsync");
  double *U0 = L > 0 ? h->Ulev(0) : Ub, *V0 = L > 0 ? h->Vlev(0) : Vb;
  cudaError_t e = cudaSuccess;
  if (rc == HODLR_OK) {
    e = launch_rand_block(su, nl, m, r, 0.0, U0, n, s);
    if (e == cudaSuccess) e = launch_rand_block(sv, nl, m, r, 0.0, V0, n, s);
    if (e == cudaSuccess) e = launch_rand_block(sd, nl, m, 1, offset, Dg, n, s);
    if (e == cudaSuccess) e = launch_seeded_leaves(U0, V0, Dg, n, m, r, nl, h->D, s);
    for (int l = 1; l < L && e == cudaSuccess; ++l) {  // every level has the same U and V
      e = cudaMemcpyAsync(h->Ulev(l), U0, sizeof(double) * n * r, cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(h->Vlev(l), V0, sizeof(double) * n * r, cudaMemcpyDeviceToDevice, s);
    }
    if (e == cudaSuccess && L > 0) e = launch_fill(h->s, (long long)L * r, 1.0, s);
  }
  for (void *p : {(void *)su, (void *)sv, (void *)sd, (void *)Dg, (void *)Ub, (void *)Vb})
    if (p) cudaFreeAsync(p, s);
  CKS(rc);
  CK(e);
  for (int l = 0; l < L; ++l) {
    h->has_level[l] = 1;
    CKS(prepare_level(h, l));
  }
  h->has_D = true;
  h->leaves_prefactored = false;
  CKS(prepare_leaves(h));
  h->factored = false;
  CK(cudaStreamSynchronize(s));
  return HODLR_OK;
}

int hodlr_set_uvd(hodlr_handle h, const double *U, int64_t ldu, const double *V, int64_t ldv, const double *Dg) {
  if (!h || !U || !V || !Dg) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  CKS(join_prep(h));  // the inputs are rewritten: set-time preparation still reading them ends first
  if (ldu < h->n || ldv < h->n) return set_err(HODLR_ERR_INVALID_ARG, "ld < n");
  std::fill(h->vsrc.begin(), h->vsrc.end(), nullptr);
  const long long n = h->n;
  const int m = h->m, L = h->L, r = h->r;
  cudaStream_t s = h->st;
  if (L == 0) return set_err(HODLR_ERR_INVALID_ARG, "hodlr_set_uvd needs levels >= 1");
  // level 0 holds the device copy of U / V; the other levels repeat it
  CK(cudaMemcpy2DAsync(h->Ulev(0), sizeof(double) * n, U, sizeof(double) * ldu, sizeof(double) * n, r,
                       cudaMemcpyDefault, s));
  CK(cudaMemcpy2DAsync(h->Vlev(0), sizeof(double) * n, V, sizeof(double) * ldv, sizeof(double) * n, r,
                       cudaMemcpyDefault, s));
  for (int l = 1; l < L; ++l) {
    CK(cudaMemcpyAsync(h->Ulev(l), h->Ulev(0), sizeof(double) * n * r, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(h->Vlev(l), h->Vlev(0), sizeof(double) * n * r, cudaMemcpyDeviceToDevice, s));
  }
  CK(launch_fill(h->s, (long long)L * r, 1.0, s));
  // leaf blocks K_i = U_i V_i^T + diag(D_i) (DenseBlockTask)
  double *dD = nullptr;
  CK(cudaMallocAsync(&dD, sizeof(double) * n, s));
  CK(cudaMemcpyAsync(dD, Dg, sizeof(double) * n, cudaMemcpyDefault, s));
  CK(cudaMemsetAsync(h->D, 0, sizeof(double) * h->nleaf * m * m, s));
  UpdateArgs ua{};
  ua.A = h->Ulev(0);
  ua.lda = n;
  ua.a_bstride = m;
  ua.B = h->Vlev(0);
  ua.ldb = n;
  ua.b_s1 = 2LL * m;
  ua.b_s2 = m;
  ua.b_trans = 1;
  ua.C = h->D;
  ua.ldc = m;
  ua.c_bstride = (long long)m * m;
  ua.M = m;
  ua.N = m;
  ua.K = r;
  ua.nbatch = h->nleaf;
  ua.alpha = 1.0;
  CK(launch_update_nn<double>(ua, s));
  CK(launch_add_leaf_diag(h->D, dD, m, h->nleaf, s));
  CK(cudaFreeAsync(dD, s));
  for (int l = 0; l < L; ++l) {
    h->has_level[l] = 1;
    CKS(prepare_level(h, l));
  }
  h->has_D = true;
  h->leaves_prefactored = false;
  CKS(prepare_leaves(h));
  h->factored = false;
  CK(cudaStreamSynchronize(s));
  return HODLR_OK;
}

}  // extern "C"

// ------------------------------------------------------ component entry points
// Short-lived device scratch for the component calls below.
struct Scratch {
  std::vector<void *> p;
  ~Scratch() {
    for (void *q : p) cudaFree(q);
  }
  template <typename T> T *get(size_t count) {
    void *q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * (count ? count : 1)) != cudaSuccess) return nullptr;
    p.push_back(q);
    return static_cast<T *>(q);
  }
};

extern "C" {

int hodlr_gemm_reduce(int nrow, int nPart, int ncolV, int ncolU, const double *V, int64_t ldv, const double *U,
                      int64_t ldu, double *W, int64_t ldw) {
  if (!V || !U || !W || nPart < 1 || nrow % nPart || ncolV < 1 || ncolV > 64 || ncolU < 1 || ldv < nrow ||
      ldu < nrow || ldw < (int64_t)nPart * ncolV)
    return set_err(HODLR_ERR_INVALID_ARG, "gemm_reduce: bad arguments");
  const long long rows = nrow / nPart;
  Scratch sc;
  double *out = sc.get<double>((size_t)nPart * ncolV * ncolU);
  double *work = sc.get<double>(reduce_workspace_doubles(rows, nPart, ncolV, ncolU, 8));
  if (!out || !work) return set_err(HODLR_ERR_OUT_OF_MEMORY, "gemm_reduce: scratch");
  CK(launch_reduce_tn<double>(V, ldv, U, ldu, rows, nPart, ncolV, ncolU, out, work, nullptr, 0));
  for (int p = 0; p < nPart; ++p)  // block p (ncolV x ncolU, ld ncolV) -> rows p*ncolV of W
    CK(cudaMemcpy2DAsync(W + (long long)p * ncolV, sizeof(double) * ldw, out + (long long)p * ncolV * ncolU,
                         sizeof(double) * ncolV, sizeof(double) * ncolV, ncolU, cudaMemcpyDeviceToDevice, 0));
  CK(cudaStreamSynchronize(0));
  return HODLR_OK;
}

int hodlr_gemm_broadcast(int nrow, int nPart, int nBlock, int K, int N, double alpha, const double *U, int64_t ldu,
                         const double *Vb, int64_t ldvb, double beta, double *W, int64_t ldw) {
  if (!U || !Vb || !W || nPart < 1 || nBlock < 1 || nPart % nBlock || nrow % nPart || K < 1 || N < 1 ||
      ldu < nrow || ldw < nrow || ldvb < (int64_t)nBlock * K)
    return set_err(HODLR_ERR_INVALID_ARG, "gemm_broadcast: bad arguments");
  const long long rows = nrow / nPart;
  const int per = nPart / nBlock;  // row partitions sharing one block of Vb
  if (beta != 1.0) CK(launch_axpy(W, ldw, W, ldw, nrow, N, beta, false, nullptr, 0));
  for (int blk = 0; blk < nBlock; ++blk) {
    UpdateArgs ua{};
    ua.A = U + (long long)blk * per * rows;
    ua.lda = ldu;
    ua.a_bstride = rows;
    ua.B = Vb + (long long)blk * K;
    ua.ldb = ldvb;
    ua.C = W + (long long)blk * per * rows;
    ua.ldc = ldw;
    ua.c_bstride = rows;
    ua.M = (int)rows;
    ua.N = N;
    ua.K = K;
    ua.nbatch = per;
    ua.alpha = alpha;
    CK(launch_update_nn<double>(ua, 0));
  }
  CK(cudaStreamSynchronize(0));
  return HODLR_OK;
}

int hodlr_node_solve(int nnode, int r, int nrhs, const double *VTu, int64_t ldu, double *VTd, int64_t ldd) {
  if (!VTu || !VTd || nnode < 1 || r < 1 || r > 64 || nrhs < 1 || ldu < 2LL * r * nnode || ldd < 2LL * r * nnode)
    return set_err(HODLR_ERR_INVALID_ARG, "node_solve: bad arguments");
  const int ct = nrhs + r;
  Scratch sc;
  double *Tb = sc.get<double>((size_t)2 * nnode * r * ct);
  double *lu = sc.get<double>((size_t)nnode * 4 * r * r);
  double *inv = sc.get<double>((size_t)nnode * 4 * r * r);
  double *eta = sc.get<double>((size_t)nnode * 2 * r * nrhs);
  int *piv = sc.get<int>((size_t)nnode * 2 * r);
  DevStatus *st = sc.get<DevStatus>(1);
  if (!Tb || !lu || !inv || !eta || !piv || !st) return set_err(HODLR_ERR_OUT_OF_MEMORY, "node_solve: scratch");
  CK(cudaMemsetAsync(st, 0, sizeof(DevStatus), 0));
  // child c = 2p + h: T_c = [VTd rows | VTu rows] of half h of node p
  for (int c = 0; c < 2 * nnode; ++c) {
    double *T = Tb + (long long)c * r * ct;
    CK(cudaMemcpy2DAsync(T, sizeof(double) * r, VTd + (long long)c * r, sizeof(double) * ldd, sizeof(double) * r,
                         nrhs, cudaMemcpyDeviceToDevice, 0));
    CK(cudaMemcpy2DAsync(T + (long long)nrhs * r, sizeof(double) * r, VTu + (long long)c * r, sizeof(double) * ldu,
                         sizeof(double) * r, r, cudaMemcpyDeviceToDevice, 0));
  }
  CapFactorArgs cf{};
  cf.Tb = Tb;
  cf.tb_stride = (long long)r * ct;
  cf.ucol = nrhs;
  cf.cap_lu = lu;
  cf.cap_ipiv = piv;
  cf.sinv = inv;
  cf.r = r;
  cf.nnode = nnode;
  cf.st = st;
  CK(launch_cap_factor(cf, 0));
  CapApplyArgs ca{};
  ca.Tb = Tb;
  ca.tb_stride = (long long)r * ct;
  ca.sinv = inv;
  ca.eta = eta;
  ca.r = r;
  ca.C = nrhs;
  ca.nnode = nnode;
  CK(launch_cap_apply(ca, 0));
  for (int p = 0; p < nnode; ++p)  // eta_p (2r x nrhs, ld 2r) -> rows [2r p, 2r (p+1)) of VTd
    CK(cudaMemcpy2DAsync(VTd + (long long)p * 2 * r, sizeof(double) * ldd, eta + (long long)p * 2 * r * nrhs,
                         sizeof(double) * 2 * r, sizeof(double) * 2 * r, nrhs, cudaMemcpyDeviceToDevice, 0));
  DevStatus hs{};
  CK(cudaMemcpy(&hs, st, sizeof(DevStatus), cudaMemcpyDeviceToHost));
  if (hs.code) return set_err(hs.code, "node_solve: singular capacitance system");
  return HODLR_OK;
}

}  // extern "C"

// =========================================================== ragged batches
// Systems that share (leaf, rank) are stacked, largest first, into one
// forest: a handle whose level l holds the blocks of every tree tall enough
// to have it, so each sweep step is one launch over all of them.  Each forest
// runs on its own stream; a batch factorisation or solve forks from the
// batch stream into the forests' streams and joins back, and from the second
// call on it is one CUDA graph launch.
struct BatchMember {
  int forest = 0;
  long long row_off = 0;  // first row of the system in its forest
  int slot0 = 0;          // forest level that holds the system's level 0
  bool has_D = false;
  std::vector<char> has_level;
};

struct BatchForest {
  hodlr_ctx *h = nullptr;
  std::vector<int> ids;          // member systems in stacking order
  long long maxn = 0;
  double *Bg = nullptr;          // stacked right-hand sides, n x kmax
  RhsCopy *tab_host = nullptr;   // pinned; read by a graph memcpy node each solve
  RhsCopy *tab_dev = nullptr;
  cudaEvent_t join = nullptr;
};

struct hodlr_batch_ctx {
  hodlr_batch_desc d{};
  std::vector<hodlr_system> sys;
  std::vector<BatchMember> mem;
  std::vector<BatchForest> forests;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  cudaEvent_t fork = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  GraphEntry factor_graph, solve_graph;
  int factor_runs = 0, solve_runs = 0;
  bool factored = false;
  float factor_ms = 0.f, solve_ms = 0.f;
};

static void free_batch(hodlr_batch_ctx *b) {
  if (!b) return;
  if (b->st) cudaStreamSynchronize(b->st);
  for (GraphEntry *g : {&b->factor_graph, &b->solve_graph})
    if (g->exec) cudaGraphExecDestroy(g->exec);
  for (auto &f : b->forests) {
    if (f.h) cudaStreamSynchronize(f.h->st);
    if (f.tab_host) cudaFreeHost(f.tab_host);
    if (f.join) cudaEventDestroy(f.join);
    free_ctx(f.h);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  for (auto &e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->own_stream && b->st) cudaStreamDestroy(b->st);
  delete b;
}

// Eager on the first call, then captured once into a graph and replayed.
template <typename F>
static int batch_graphed(hodlr_batch_ctx *b, GraphEntry &g, int &runs, F fn) {
  if (runs == 0) {
    ++runs;
    return fn();
  }
  if (!g.exec) {
    const long long before = g_launches.load();
    CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    int rc = fn();
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(b->st, &graph);
    if (rc != HODLR_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    CK(ce);
    cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ie);
    g.kernels = g_launches.load() - before;
    g_launches.fetch_sub(g.kernels);
  }
  g_launches.fetch_add(g.kernels);
  CK(cudaGraphLaunch(g.exec, b->st));
  ++runs;
  return HODLR_OK;
}

// Run body(forest) on every forest's stream, forked from and joined back
// into the batch stream.
template <typename F>
static int batch_forked(hodlr_batch_ctx *b, F body) {
  CK(cudaEventRecord(b->fork, b->st));
  for (auto &f : b->forests) {
    CK(cudaStreamWaitEvent(f.h->st, b->fork, 0));
    {
      TuningScope tscope(&f.h->tune);
      CKS(body(f));
    }
    CK(cudaEventRecord(f.join, f.h->st));
    CK(cudaStreamWaitEvent(b->st, f.join, 0));
  }
  return HODLR_OK;
}

// The system that owns row `row` of forest f (or -1).
static int batch_owner(const hodlr_batch_ctx *b, const BatchForest &f, long long row) {
  for (int id : f.ids) {
    const BatchMember &mb = b->mem[id];
    if (row >= mb.row_off && row < mb.row_off + b->sys[id].n) return id;
  }
  return -1;
}

// Read every forest's device status; on an error name the system.
static int batch_status(hodlr_batch_ctx *b, hodlr_solve_info *info) {
  int first = HODLR_OK;
  std::string msg;
  for (auto &f : b->forests) {
    hodlr_ctx *h = f.h;
    CK(cudaMemcpy(h->hst, h->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost));
    const DevStatus s = *h->hst;
    if (info)
      for (int id : f.ids) {
        info[id].status = s.code;
        info[id].iterations = s.iters;
        info[id].bad_index = -1;
        info[id].rel_residual = -1.0;
      }
    if (s.code == HODLR_OK) continue;
    long long row = s.index;  // a row for leaf / input errors, a node for capacitance errors
    if (s.code == HODLR_ERR_SINGULAR_LEAF) row = s.index * h->m;
    if (s.code == HODLR_ERR_SINGULAR_CAPACITANCE)
      for (int l = h->L - 1; l >= 0; --l)
        if (s.index >= h->node_base(l)) {
          row = (s.index - h->node_base(l)) * 2 * h->rows(l);
          break;
        }
    const int id = batch_owner(b, f, row);
    if (info && id >= 0) info[id].bad_index = s.index;
    if (first == HODLR_OK) {
      first = s.code;
      char buf[160];
      snprintf(buf, sizeof buf, "system %d: error %d (forest index %lld)", id, s.code, s.index);
      msg = buf;
    }
  }
  if (first != HODLR_OK) return set_err(first, msg);
  return HODLR_OK;
}

extern "C" {

int hodlr_batch_create(const hodlr_batch_desc *desc, hodlr_batch *out) {
  if (!desc || !out || !desc->systems || desc->count < 1)
    return set_err(HODLR_ERR_INVALID_ARG, "batch: null argument or empty batch");
  *out = nullptr;
  const hodlr_batch_desc &d = *desc;
  std::map<std::pair<int, int>, std::vector<int>> groups;
  for (int i = 0; i < d.count; ++i) {
    const hodlr_system &s = d.systems[i];
    if (s.leaf < 1 || s.levels < 0 || s.levels > 24 || s.n != ((int64_t)s.leaf << s.levels) || s.nrhs < 1 ||
        (s.levels > 0 && (s.rank < 1 || s.rank > 64))) {
      char buf[128];
      snprintf(buf, sizeof buf, "batch: system %d needs n = leaf * 2^levels, rank in [1, 64], nrhs >= 1", i);
      return set_err(HODLR_ERR_INVALID_ARG, buf);
    }
    if (s.levels > 0) groups[{s.leaf, s.rank}].push_back(i);
  }
  // one-leaf systems (no levels) join a forest of their leaf size, if any
  for (int i = 0; i < d.count; ++i) {
    const hodlr_system &s = d.systems[i];
    if (s.levels > 0) continue;
    auto it = groups.lower_bound({s.leaf, 0});
    if (it != groups.end() && it->first.first == s.leaf)
      it->second.push_back(i);
    else
      groups[{s.leaf, 0}].push_back(i);
  }
  hodlr_batch_ctx *b = new hodlr_batch_ctx();
  b->d = d;
  b->sys.assign(d.systems, d.systems + d.count);
  b->d.systems = nullptr;
  b->mem.resize(d.count);
  auto fail = [&](int code, const std::string &m) {
    free_batch(b);
    return set_err(code, m);
  };
  if (d.stream) {
    b->st = (cudaStream_t)d.stream;
  } else {
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess)
      return fail(HODLR_ERR_CUDA, "batch: stream");
    b->own_stream = true;
  }
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
    return fail(HODLR_ERR_CUDA, "batch: event");
  for (auto &e : b->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(HODLR_ERR_CUDA, "batch: event");
  for (auto &g : groups) {
    std::vector<int> ids = g.second;
    std::stable_sort(ids.begin(), ids.end(),
                     [&](int a, int c) { return b->sys[a].levels > b->sys[c].levels; });
    hodlr_desc fd{};
    fd.leaf = g.first.first;
    fd.rank = std::max(1, g.first.second);
    fd.levels = b->sys[ids[0]].levels;
    fd.n = 0;
    fd.nrhs_max = 1;
    std::vector<int> lv;
    for (int id : ids) {
      fd.n += b->sys[id].n;
      fd.nrhs_max = std::max(fd.nrhs_max, b->sys[id].nrhs);
      lv.push_back(b->sys[id].levels);
    }
    fd.precision = d.precision;
    fd.residual = d.residual;
    fd.refine_tol = d.refine_tol;
    fd.refine_max_iter = d.refine_max_iter;
    int rc = check_common(fd);
    if (rc != HODLR_OK) return fail(rc, hodlr_last_error_string());
    if (fd.n / fd.leaf > (1LL << 30)) return fail(HODLR_ERR_INVALID_ARG, "batch: too many leaves in one forest");
    BatchForest f;
    rc = create_ctx(fd, lv, &f.h);
    if (rc != HODLR_OK) return fail(rc, hodlr_last_error_string());
    b->forests.push_back(f);
    BatchForest &F = b->forests.back();
    F.ids = ids;
    long long off = 0;
    for (int id : ids) {
      BatchMember &mb = b->mem[id];
      mb.forest = (int)b->forests.size() - 1;
      mb.row_off = off;
      mb.slot0 = fd.levels - b->sys[id].levels;
      mb.has_level.assign(b->sys[id].levels, 0);
      off += b->sys[id].n;
      F.maxn = std::max<long long>(F.maxn, b->sys[id].n);
    }
    cudaError_t e = cudaSuccess;
    F.Bg = F.h->alloc<double>((size_t)fd.n * fd.nrhs_max, e);
    if (e != cudaSuccess) return fail(HODLR_ERR_OUT_OF_MEMORY, "batch: right-hand-side buffer");
    F.tab_dev = F.h->alloc<RhsCopy>(ids.size(), e);
    if (e != cudaSuccess) return fail(HODLR_ERR_OUT_OF_MEMORY, "batch: copy table");
    if (cudaMallocHost(&F.tab_host, sizeof(RhsCopy) * ids.size()) != cudaSuccess)
      return fail(HODLR_ERR_OUT_OF_MEMORY, "batch: pinned copy table");
    if (cudaEventCreateWithFlags(&F.join, cudaEventDisableTiming) != cudaSuccess)
      return fail(HODLR_ERR_CUDA, "batch: event");
  }
  *out = b;
  return HODLR_OK;
}

int hodlr_batch_destroy(hodlr_batch b) {
  free_batch(b);
  return HODLR_OK;
}

int hodlr_batch_set_leaf_blocks(hodlr_batch b, int i, const double *D, int64_t ld, int64_t leaf_stride) {
  if (!b || !D || i < 0 || i >= (int)b->sys.size()) return set_err(HODLR_ERR_INVALID_ARG, "batch: bad argument");
  const hodlr_system &sy = b->sys[i];
  BatchMember &mb = b->mem[i];
  hodlr_ctx *h = b->forests[mb.forest].h;
  const int m = sy.leaf;
  if (ld < m) return set_err(HODLR_ERR_INVALID_ARG, "batch: ld < leaf size");
  const long long mm = (long long)m * m, leaf0 = mb.row_off / m, nl = sy.n / m;
  double *dst = h->D + leaf0 * mm;
  if (ld == m && leaf_stride == mm) {
    CK(cudaMemcpyAsync(dst, D, sizeof(double) * mm * nl, cudaMemcpyDefault, h->st));
  } else {
    for (int j = 0; j < m; ++j)
      CK(cudaMemcpy2DAsync(dst + (long long)j * m, sizeof(double) * mm, D + (long long)j * ld,
                           sizeof(double) * leaf_stride, sizeof(double) * m, nl, cudaMemcpyDefault, h->st));
  }
  CKS(prepare_leaves(h, leaf0, nl));
  mb.has_D = true;
  b->factored = false;
  CK(cudaStreamSynchronize(h->st));
  return HODLR_OK;
}

int hodlr_batch_set_lowrank(hodlr_batch b, int i, int level, const double *U, int64_t ldu, const double *V,
                            int64_t ldv, const double *s) {
  if (!b || !U || !V || i < 0 || i >= (int)b->sys.size()) return set_err(HODLR_ERR_INVALID_ARG, "batch: bad argument");
  const hodlr_system &sy = b->sys[i];
  BatchMember &mb = b->mem[i];
  hodlr_ctx *h = b->forests[mb.forest].h;
  if (level < 0 || level >= sy.levels) return set_err(HODLR_ERR_INVALID_ARG, "batch: level out of range");
  if (ldu < sy.n || ldv < sy.n) return set_err(HODLR_ERR_INVALID_ARG, "batch: ld < n");
  const int slot = mb.slot0 + level, r = h->r;
  double *Ud = h->Ulev(slot) + mb.row_off, *Vd = h->Vlev(slot) + mb.row_off;
  CK(cudaMemcpy2DAsync(Ud, sizeof(double) * h->n, U, sizeof(double) * ldu, sizeof(double) * sy.n, r,
                       cudaMemcpyDefault, h->st));
  CK(cudaMemcpy2DAsync(Vd, sizeof(double) * h->n, V, sizeof(double) * ldv, sizeof(double) * sy.n, r,
                       cudaMemcpyDefault, h->st));
  if (s) {
    CK(cudaMemcpyAsync(h->sfold, s, sizeof(double) * r, cudaMemcpyDefault, h->st));
    CK(launch_scale_cols(Vd, h->n, sy.n, r, h->sfold, h->st));
  }
  CKS(prepare_level(h, slot, mb.row_off, sy.n));
  mb.has_level[level] = 1;
  b->factored = false;
  CK(cudaStreamSynchronize(h->st));
  return HODLR_OK;
}

int hodlr_batch_generate(hodlr_batch b, uint64_t seed, double shift, double *const *B, const int64_t *ldb) {
  if (!b) return set_err(HODLR_ERR_INVALID_ARG, "batch: null handle");
  for (int i = 0; i < (int)b->sys.size(); ++i) {
    const hodlr_system &sy = b->sys[i];
    BatchMember &mb = b->mem[i];
    hodlr_ctx *h = b->forests[mb.forest].h;
    const int m = sy.leaf, r = h->r;
    const unsigned long long si = seed + (unsigned long long)i;
    const long long leaf0 = mb.row_off / m, nl = sy.n / m;
    CK(launch_gen_leaves(h->D + leaf0 * m * m, m, (int)nl, si, shift, h->st));
    CKS(prepare_leaves(h, leaf0, nl));
    mb.has_D = true;
    for (int l = 0; l < sy.levels; ++l) {
      const int slot = mb.slot0 + l;
      const long long rows = sy.n >> (l + 1);
      for (int w = 0; w < 2; ++w) {
        double *X = (w == 0 ? h->Ulev(slot) : h->Vlev(slot)) + mb.row_off;
        CK(launch_gaussian(X, h->n, sy.n, r, si, 0x100ull + 2ull * l + w, 1.0 / std::sqrt((double)rows), h->st));
      }
      CKS(prepare_level(h, slot, mb.row_off, sy.n));
      mb.has_level[l] = 1;
    }
    if (B && B[i]) {
      if (!ldb || ldb[i] < sy.n) return set_err(HODLR_ERR_INVALID_ARG, "batch: ldb < n");
      CK(launch_gaussian(B[i], ldb[i], sy.n, sy.nrhs, si, 0xBull, 1.0, h->st));
    }
  }
  for (auto &f : b->forests) CK(cudaStreamSynchronize(f.h->st));
  b->factored = false;
  return HODLR_OK;
}

int hodlr_batch_factor(hodlr_batch b) {
  if (!b) return set_err(HODLR_ERR_INVALID_ARG, "batch: null handle");
  for (int i = 0; i < (int)b->sys.size(); ++i) {
    const BatchMember &mb = b->mem[i];
    bool ok = mb.has_D;
    for (char c : mb.has_level) ok = ok && c;
    if (!ok) {
      char buf[96];
      snprintf(buf, sizeof buf, "batch: system %d has unset leaf blocks or levels", i);
      return set_err(HODLR_ERR_NOT_FACTORED, buf);
    }
  }
  b->factored = false;
  CK(cudaEventRecord(b->ev[0], b->st));
  int rc = batch_graphed(b, b->factor_graph, b->factor_runs, [&]() -> int {
    return batch_forked(b, [&](BatchForest &f) -> int {
      CKS(reset_status(f.h));
      if (f.h->mixed) return factor_sweep<float>(f.h);
      return factor_sweep<double>(f.h);
    });
  });
  CKS(rc);
  CK(cudaEventRecord(b->ev[1], b->st));
  CK(cudaStreamSynchronize(b->st));
  CKS(batch_status(b, nullptr));
  cudaEventElapsedTime(&b->factor_ms, b->ev[0], b->ev[1]);
  for (auto &f : b->forests) f.h->factored = true;
  b->factored = true;
  return HODLR_OK;
}

int hodlr_batch_solve(hodlr_batch b, double *const *B, const int64_t *ldb, hodlr_solve_info *info) {
  if (!b || !B || !ldb) return set_err(HODLR_ERR_INVALID_ARG, "batch: null argument");
  if (!b->factored) return set_err(HODLR_ERR_NOT_FACTORED, "batch: call hodlr_batch_factor first");
  for (auto &f : b->forests)
    for (size_t q = 0; q < f.ids.size(); ++q) {
      const int id = f.ids[q];
      const hodlr_system &sy = b->sys[id];
      if (!B[id] || ldb[id] < sy.n) return set_err(HODLR_ERR_INVALID_ARG, "batch: null B[i] or ldb[i] < n_i");
      RhsCopy t{};
      t.ext = B[id];
      t.ld = ldb[id];
      t.row_off = b->mem[id].row_off;
      t.n = sy.n;
      t.k = sy.nrhs;
      f.tab_host[q] = t;
    }
  CK(cudaEventRecord(b->ev[2], b->st));
  int rc = batch_graphed(b, b->solve_graph, b->solve_runs, [&]() -> int {
    return batch_forked(b, [&](BatchForest &f) -> int {
      hodlr_ctx *h = f.h;
      const int nid = (int)f.ids.size(), k = h->kmax;
      CKS(reset_status(h));
      CK(cudaMemcpyAsync(f.tab_dev, f.tab_host, sizeof(RhsCopy) * nid, cudaMemcpyHostToDevice, h->st));
      CK(launch_gather_rhs(f.tab_dev, nid, f.maxn, f.Bg, h->n, k, h->st));
      CK(launch_check_finite(f.Bg, h->n, h->n, k, h->dst, h->st));
      if (h->mixed)
        CKS(mixed_solve(h, f.Bg, h->n, k, false));
      else
        CKS(solve_sweep<double>(h, f.Bg, h->n, k, false, nullptr));
      CK(launch_scatter_rhs(f.tab_dev, nid, f.maxn, f.Bg, h->n, k, h->st));
      return HODLR_OK;
    });
  });
  CKS(rc);
  CK(cudaEventRecord(b->ev[3], b->st));
  CK(cudaStreamSynchronize(b->st));
  cudaEventElapsedTime(&b->solve_ms, b->ev[2], b->ev[3]);
  int st = batch_status(b, info);
  // per-system relative residuals of the refinement (mixed mode)
  if (info && b->d.precision == HODLR_PREC_MIXED)
    for (auto &f : b->forests) {
      hodlr_ctx *h = f.h;
      const size_t cnt = (size_t)h->nsys * h->kmax;
      std::vector<double> nb(2 * cnt);
      CK(cudaMemcpy(nb.data(), h->norms, sizeof(double) * 2 * cnt, cudaMemcpyDeviceToHost));
      for (size_t q = 0; q < f.ids.size(); ++q) {
        const int id = f.ids[q];
        double rel = 0.0;
        for (int j = 0; j < b->sys[id].nrhs; ++j) {
          const double bn = nb[(size_t)j * h->nsys + q], rn = nb[cnt + (size_t)j * h->nsys + q];
          rel = std::max(rel, rn / (bn > 0.0 ? bn : 1.0));
        }
        info[id].rel_residual = rel;
      }
    }
  if (st != HODLR_OK) return st;
  if (b->d.precision == HODLR_PREC_MIXED)
    for (auto &f : b->forests)
      if (!f.h->hst->done) {
        if (info)
          for (int id : f.ids) info[id].status = HODLR_ERR_NOT_CONVERGED;
        return set_err(HODLR_ERR_NOT_CONVERGED, "batch: refinement did not reach the tolerance");
      }
  return HODLR_OK;
}

int hodlr_batch_stats(hodlr_batch b, int *nforests, double *factor_ms, double *solve_ms) {
  if (!b) return set_err(HODLR_ERR_INVALID_ARG, "batch: null handle");
  if (nforests) *nforests = (int)b->forests.size();
  if (factor_ms) *factor_ms = b->factor_ms;
  if (solve_ms) *solve_ms = b->solve_ms;
  return HODLR_OK;
}

}  // extern "C"

// ================================================================ autotuner
// Coordinate search over the tunable launch shapes (split-K target of the
// row reductions, FP32 update tile rows), timing complete factor + solve
// sweeps on the handle's own inputs with a seeded scratch right-hand side.
static const int kRedCands[] = {2, 4, 8};
static const int kUpdCands[] = {0, 64};
static const int kCapWarpCands[] = {0, 8, 16};
static const int kUpdTcCands[] = {0, 1, 2};

template <typename Measure>
static int tune_search(Tuning &cur, double &cur_ms, Measure measure) {
  CKS(measure(cur, cur_ms));
  for (int red : kRedCands) {
    if (red == cur.red_ctas_per_sm) continue;
    Tuning t = cur;
    t.red_ctas_per_sm = red;
    double ms = 0.0;
    CKS(measure(t, ms));
    if (ms < cur_ms) cur = t, cur_ms = ms;
  }
  for (int bm : kUpdCands) {
    if (bm == cur.upd_bm) continue;
    Tuning t = cur;
    t.upd_bm = bm;
    double ms = 0.0;
    CKS(measure(t, ms));
    if (ms < cur_ms) cur = t, cur_ms = ms;
  }
  for (int sh : kUpdTcCands) {
    if (sh == cur.upd_tc_shape) continue;
    Tuning t = cur;
    t.upd_tc_shape = sh;
    double ms = 0.0;
    CKS(measure(t, ms));
    if (ms < cur_ms) cur = t, cur_ms = ms;
  }
  for (int w : kCapWarpCands) {
    if (w == cur.cap_warps) continue;
    Tuning t = cur;
    t.cap_warps = w;
    double ms = 0.0;
    CKS(measure(t, ms));
    if (ms < cur_ms) cur = t, cur_ms = ms;
  }
  for (int la : {0, 1}) {
    if (la == cur.leaf_apply) continue;
    Tuning t = cur;
    t.leaf_apply = la;
    double ms = 0.0;
    CKS(measure(t, ms));
    if (ms < cur_ms) cur = t, cur_ms = ms;
  }
  return HODLR_OK;
}

static bool valid_tuning(const hodlr_tuning &t) {
  return (t.red_ctas_per_sm == 2 || t.red_ctas_per_sm == 4 || t.red_ctas_per_sm == 8) &&
         (t.update_tile_rows == 0 || t.update_tile_rows == 64 || t.update_tile_rows == 128) &&
         (t.cap_warps == 0 || t.cap_warps == 8 || t.cap_warps == 16 || t.cap_warps == 32) &&
         t.update_tc_shape >= 0 && t.update_tc_shape <= 2 && (t.leaf_apply == 0 || t.leaf_apply == 1);
}

extern "C" {

int hodlr_set_tuning(hodlr_handle h, const hodlr_tuning *t) {
  if (!h || !t || !valid_tuning(*t)) return set_err(HODLR_ERR_INVALID_ARG, "bad tuning");
  h->tune.red_ctas_per_sm = t->red_ctas_per_sm;
  h->tune.upd_bm = t->update_tile_rows == 128 ? 0 : t->update_tile_rows;
  h->tune.cap_warps = t->cap_warps;
  h->tune.upd_tc_shape = t->update_tc_shape;
  h->tune.leaf_apply = t->leaf_apply;
  clear_graphs(h);
  h->factored = false;
  return HODLR_OK;
}

int hodlr_get_tuning(hodlr_handle h, hodlr_tuning *t) {
  if (!h || !t) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  t->red_ctas_per_sm = h->tune.red_ctas_per_sm;
  t->update_tile_rows = h->tune.upd_bm;
  t->cap_warps = h->tune.cap_warps;
  t->update_tc_shape = h->tune.upd_tc_shape;
  t->leaf_apply = h->tune.leaf_apply;
  t->ms = -1.0;
  return HODLR_OK;
}

int hodlr_autotune(hodlr_handle h, int nrhs, hodlr_tuning *best) {
  if (!h) return set_err(HODLR_ERR_INVALID_ARG, "null handle");
  if (nrhs < 1 || nrhs > h->kmax) return set_err(HODLR_ERR_INVALID_ARG, "nrhs out of range");
  if (!h->has_D) return set_err(HODLR_ERR_NOT_FACTORED, "leaf blocks not set");
  for (int l = 0; l < h->L; ++l)
    if (!h->has_level[l]) return set_err(HODLR_ERR_NOT_FACTORED, "low-rank level not set");
  const long long n = h->n;
  double *B = nullptr;
  CK(cudaMalloc(&B, sizeof(double) * n * nrhs));
  auto measure = [&](const Tuning &t, double &ms) -> int {
    h->tune = t;
    clear_graphs(h);
    for (int rep = 0; rep < 3; ++rep) {  // eager, captured, replayed: the last is timed
      CK(launch_gaussian(B, n, n, nrhs, 0x5eedull, 0x7ull, 1.0, h->st));
      CKS(hodlr_factor(h));
      hodlr_solve_info info;
      const int rc = solve_impl(h, B, n, nrhs, &info, false);
      if (rc != HODLR_OK && rc != HODLR_ERR_NOT_CONVERGED) return rc;
    }
    ms = (double)h->factor_ms + (double)h->solve_ms;
    return HODLR_OK;
  };
  Tuning cur = h->tune;
  double cur_ms = 0.0;
  int rc = tune_search(cur, cur_ms, measure);
  cudaFree(B);
  CKS(rc);
  h->tune = cur;
  clear_graphs(h);
  h->factored = false;
  CKS(hodlr_factor(h));  // leave the handle factored with the chosen shapes
  if (best) {
    best->red_ctas_per_sm = cur.red_ctas_per_sm;
    best->update_tile_rows = cur.upd_bm;
    best->cap_warps = cur.cap_warps;
    best->update_tc_shape = cur.upd_tc_shape;
    best->leaf_apply = cur.leaf_apply;
    best->ms = cur_ms;
  }
  return HODLR_OK;
}

int hodlr_batch_autotune(hodlr_batch b, hodlr_tuning *per_forest, int capacity) {
  if (!b) return set_err(HODLR_ERR_INVALID_ARG, "batch: null handle");
  for (int i = 0; i < (int)b->sys.size(); ++i) {
    bool ok = b->mem[i].has_D;
    for (char c : b->mem[i].has_level) ok = ok && c;
    if (!ok) return set_err(HODLR_ERR_NOT_FACTORED, "batch: inputs not set");
  }
  for (size_t fi = 0; fi < b->forests.size(); ++fi) {
    hodlr_ctx *h = b->forests[fi].h;
    const long long n = h->n;
    const int k = h->kmax;
    double *B = nullptr;
    CK(cudaMalloc(&B, sizeof(double) * n * k));
    auto measure = [&](const Tuning &t, double &ms) -> int {
      h->tune = t;
      TuningScope tscope(&h->tune);
      for (int rep = 0; rep < 2; ++rep) {  // the second run is timed
        CK(launch_gaussian(B, n, n, k, 0x5eedull, 0x7ull, 1.0, h->st));
        CK(cudaEventRecord(b->ev[0], h->st));
        CKS(reset_status(h));
        CKS(h->mixed ? factor_sweep<float>(h) : factor_sweep<double>(h));
        CKS(h->mixed ? mixed_solve(h, B, n, k, false) : solve_sweep<double>(h, B, n, k, false, nullptr));
        CK(cudaEventRecord(b->ev[1], h->st));
        CK(cudaStreamSynchronize(h->st));
      }
      float f = 0.f;
      CK(cudaEventElapsedTime(&f, b->ev[0], b->ev[1]));
      ms = f;
      return HODLR_OK;
    };
    Tuning cur = h->tune;
    double cur_ms = 0.0;
    int rc = tune_search(cur, cur_ms, measure);
    cudaFree(B);
    CKS(rc);
    h->tune = cur;
    if (per_forest && (int)fi < capacity) {
      per_forest[fi].red_ctas_per_sm = cur.red_ctas_per_sm;
      per_forest[fi].update_tile_rows = cur.upd_bm;
      per_forest[fi].cap_warps = cur.cap_warps;
      per_forest[fi].update_tc_shape = cur.upd_tc_shape;
      per_forest[fi].leaf_apply = cur.leaf_apply;
      per_forest[fi].ms = cur_ms;
    }
  }
  for (GraphEntry *g : {&b->factor_graph, &b->solve_graph}) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    *g = GraphEntry();
  }
  b->factor_runs = b->solve_runs = 0;
  b->factored = false;
  return (int)b->forests.size() > 0 ? HODLR_OK : HODLR_OK;
}

}  // extern "C"

// ------------------------------------------------------------- checkpoints
// A factored handle as one host byte stream: a header (descriptor, launch
// shapes, payload size and checksum), then every input and factor buffer as
// (uint64 byte count, bytes).  The input-derived copies of the mixed path
// (FP32 V, double-word and digit splits) are rebuilt from the inputs on load
// rather than stored; workspaces are not state.  No reference counterpart:
// the reference refactors on every solve (src/hmatrix.cc:49-96).
namespace {

constexpr char kCkMagic[8] = {'H', 'O', 'D', 'L', 'R', 'C', 'K', '1'};
constexpr uint32_t kCkVersion = 3;

struct CkHeader {
  char magic[8];
  uint32_t version, nbuf;
  int64_t n;
  int32_t leaf, levels, rank, nrhs_max, precision, residual;
  double refine_tol;
  int32_t refine_max_iter, flags;
  int32_t red_ctas_per_sm, update_tile_rows, cap_warps, update_tc_shape, leaf_apply, reserved;
  uint64_t payload, checksum;
};

struct CkBuf {
  void *p;
  size_t bytes;
};

// The state buffers of a plain handle, in stream order.
std::vector<CkBuf> ck_buffers(const hodlr_ctx *h) {
  const size_t n = h->n, m = h->m, L = h->L, r = h->r, nl = h->nleaf, nn = h->nnode;
  const size_t mm = m * m, nlr = n * L * r, cap = nn * 4 * r * r;
  const bool x = h->mixed;
  const size_t w = x ? 4 : 8;  // element size of the factor buffers
  void *sinv = x ? (void *)h->Sinv32 : (void *)h->Sinv;
  void *dinv = x ? (void *)h->Dinv32 : (void *)h->Dinv;
  void *lu = x ? (void *)h->LU32 : (void *)h->LU;
  void *ut = x ? (void *)h->Ut32 : (void *)h->Ut;
  return {{h->D, nl * mm * 8},         {h->U, nlr * 8},       {h->V, nlr * 8},
          {h->s, L * r * 8},           {h->ipiv, n * 4},      {h->capLU, cap * 8},
          {h->cap_ipiv, nn * 2 * r * 4}, {sinv, cap * w},     {dinv, dinv ? nl * mm * w : 0},
          {lu, nl * mm * w},           {ut, nlr * w}};
}

// Fletcher-style sum over 32-bit words (every buffer is a whole number of them).
void ck_sum(const unsigned char *p, size_t bytes, uint64_t &a, uint64_t &b) {
  const size_t nw = bytes / 4;
  for (size_t i = 0; i < nw; ++i) {
    uint32_t v;
    memcpy(&v, p + 4 * i, 4);
    a += v;
    b += a;
  }
}

}  // namespace

extern "C" {

int hodlr_checkpoint_size(hodlr_handle h, int64_t *bytes) {
  if (!h || !bytes) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  if (h->forest) return set_err(HODLR_ERR_INVALID_ARG, "batch handles have no checkpoint");
  if (!h->factored) return set_err(HODLR_ERR_NOT_FACTORED, "not factored");
  size_t total = sizeof(CkHeader);
  for (const CkBuf &b : ck_buffers(h)) total += 8 + b.bytes;
  *bytes = (int64_t)total;
  return HODLR_OK;
}

int hodlr_checkpoint_save(hodlr_handle h, void *buf, int64_t bytes) {
  int64_t need = 0;
  CKS(hodlr_checkpoint_size(h, &need));
  if (!buf) return set_err(HODLR_ERR_INVALID_ARG, "null buffer");
  CKS(join_prep(h));  // the side stream may still be writing the leaf factors
  if (bytes < need) return set_err(HODLR_ERR_INVALID_ARG, "checkpoint buffer too small");
  if (h->factored) CKS(ensure_leaf_lu(h));
  CK(cudaStreamSynchronize(h->st));
  unsigned char *out = static_cast<unsigned char *>(buf);
  unsigned char *p = out + sizeof(CkHeader);
  const std::vector<CkBuf> bufs = ck_buffers(h);
  for (const CkBuf &b : bufs) {
    const uint64_t nb = b.bytes;
    memcpy(p, &nb, 8);
    p += 8;
    if (nb) CK(cudaMemcpy(p, b.p, nb, cudaMemcpyDeviceToHost));
    p += nb;
  }
  CkHeader hd{};
  memcpy(hd.magic, kCkMagic, 8);
  hd.version = kCkVersion;
  hd.nbuf = (uint32_t)bufs.size();
  hd.n = h->d.n;
  hd.leaf = h->d.leaf;
  hd.levels = h->d.levels;
  hd.rank = h->d.rank;
  hd.nrhs_max = h->d.nrhs_max;
  hd.precision = h->d.precision;
  hd.residual = h->d.residual;
  hd.refine_tol = h->d.refine_tol;
  hd.refine_max_iter = h->d.refine_max_iter;
  hd.flags = h->d.flags;
  hd.red_ctas_per_sm = h->tune.red_ctas_per_sm;
  hd.update_tile_rows = h->tune.upd_bm;
  hd.cap_warps = h->tune.cap_warps;
  hd.update_tc_shape = h->tune.upd_tc_shape;
  hd.leaf_apply = h->tune.leaf_apply;
  hd.payload = (uint64_t)(p - out) - sizeof(CkHeader);
  uint64_t a = 1, c = 0;
  ck_sum(out + sizeof(CkHeader), hd.payload, a, c);
  hd.checksum = a ^ (c << 1);
  memcpy(out, &hd, sizeof hd);
  return HODLR_OK;
}

int hodlr_checkpoint_load(const void *buf, int64_t bytes, void *stream, hodlr_handle *out) {
  if (!buf || !out) return set_err(HODLR_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (bytes < (int64_t)sizeof(CkHeader)) return set_err(HODLR_ERR_INVALID_ARG, "checkpoint truncated");
  const unsigned char *in = static_cast<const unsigned char *>(buf);
  CkHeader hd;
  memcpy(&hd, in, sizeof hd);
  if (memcmp(hd.magic, kCkMagic, 8) != 0 || hd.version != kCkVersion)
    return set_err(HODLR_ERR_INVALID_ARG, "not a checkpoint of this library version");
  if (hd.payload > (uint64_t)bytes - sizeof(CkHeader)) return set_err(HODLR_ERR_INVALID_ARG, "checkpoint truncated");
  uint64_t a = 1, c = 0;
  ck_sum(in + sizeof(CkHeader), hd.payload, a, c);
  if ((a ^ (c << 1)) != hd.checksum) return set_err(HODLR_ERR_INVALID_ARG, "checkpoint checksum mismatch");
  hodlr_desc d{};
  d.n = hd.n;
  d.leaf = hd.leaf;
  d.levels = hd.levels;
  d.rank = hd.rank;
  d.nrhs_max = hd.nrhs_max;
  d.precision = hd.precision;
  d.residual = hd.residual;
  d.refine_tol = hd.refine_tol;
  d.refine_max_iter = hd.refine_max_iter;
  d.flags = hd.flags;
  d.stream = stream;
  hodlr_tuning t{hd.red_ctas_per_sm, hd.update_tile_rows, hd.cap_warps, hd.update_tc_shape, hd.leaf_apply, -1.0};
  if (!valid_tuning(t)) return set_err(HODLR_ERR_INVALID_ARG, "checkpoint holds unknown launch shapes");
  hodlr_handle h = nullptr;
  CKS(hodlr_create(&d, &h));
  auto fail = [&](int code, const char *msg) {
    hodlr_destroy(h);
    return set_err(code, msg);
  };
  if (hodlr_set_tuning(h, &t) != HODLR_OK) return fail(HODLR_ERR_INVALID_ARG, "checkpoint launch shapes");
  const std::vector<CkBuf> bufs = ck_buffers(h);
  if (hd.nbuf != bufs.size()) return fail(HODLR_ERR_INVALID_ARG, "checkpoint does not match its descriptor");
  const unsigned char *p = in + sizeof(CkHeader), *end = p + hd.payload;
  for (const CkBuf &b : bufs) {
    uint64_t nb = 0;
    if (end - p < 8) return fail(HODLR_ERR_INVALID_ARG, "checkpoint truncated");
    memcpy(&nb, p, 8);
    p += 8;
    if (nb != b.bytes || (uint64_t)(end - p) < nb)
      return fail(HODLR_ERR_INVALID_ARG, "checkpoint does not match its descriptor");
    if (nb && cudaMemcpy(b.p, p, nb, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(HODLR_ERR_CUDA, "checkpoint copy to the device");
    p += nb;
  }
  h->has_D = true;
  h->leaves_prefactored = false;
  std::fill(h->has_level.begin(), h->has_level.end(), (char)1);
  int rc = prepare_leaves(h);
  for (int l = 0; l < h->L && rc == HODLR_OK; ++l) rc = prepare_level(h, l);
  if (rc != HODLR_OK) {
    hodlr_destroy(h);
    return rc;
  }
  if (cudaStreamSynchronize(h->st) != cudaSuccess) return fail(HODLR_ERR_CUDA, "checkpoint preparation");
  h->factored = true;
  *out = h;
  return HODLR_OK;
}

}  // extern "C"
