"""ctypes front end of the C oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module; it is the checker, never part of the product path.

All matrices are numpy float64 arrays in Fortran (column-major) order, the
layout fastSolver2 uses throughout (src/ptr_matrix.cc:29-37).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None
_blas = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)
_i64 = ctypes.c_int64


def lib():
    """Load (building if needed) libhodlr_oracle.so."""
    global _lib
    if _lib is None:
        path = _build.ORACLE_SO
        if not os.path.exists(path):
            _build.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_seeds.argtypes = [ctypes.c_long, ctypes.c_int, _lp]
        L.orc_rand_block.argtypes = [ctypes.c_long, ctypes.c_int, ctypes.c_int, _i64, _dp, ctypes.c_int]
        L.orc_rand_matrix.argtypes = [_lp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int]
        L.orc_dense_blocks.argtypes = [_lp, _lp, _lp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, _dp, _i64]
        L.orc_idamax.argtypes = [ctypes.c_int, _dp]
        L.orc_idamax.restype = ctypes.c_int
        L.orc_dgemm.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_double, _dp, _i64, _dp, _i64, ctypes.c_double, _dp, _i64]
        L.orc_dgetrf.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _i64, _ip]
        L.orc_dgetrf.restype = ctypes.c_int
        L.orc_dgetrf2.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _i64, _ip]
        L.orc_dgetrf2.restype = ctypes.c_int
        L.orc_dgetrs.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, _dp, _i64, _ip, _dp, _i64]
        L.orc_dgesv.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _i64, _ip, _dp, _i64]
        L.orc_dgesv.restype = ctypes.c_int
        L.orc_hsolve.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i64, _dp, _dp, _dp]
        L.orc_hsolve.restype = ctypes.c_int
        L.orc_hsolve_general.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _i64,
                                         ctypes.POINTER(_dp), _i64, ctypes.POINTER(_dp), ctypes.c_int,
                                         _dp, _i64, _ip, _dp, _ip]
        L.orc_hsolve_general.restype = ctypes.c_int
        L.orc_hsolve_general_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _i64,
                                            ctypes.POINTER(_dp), _i64, ctypes.POINTER(_dp), ctypes.c_int,
                                            _dp, _i64, ctypes.c_int]
        L.orc_hsolve_general_mt.restype = ctypes.c_int
        L.orc_hodlr_matvec.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _i64,
                                       ctypes.POINTER(_dp), _i64, ctypes.POINTER(_dp), _i64,
                                       ctypes.POINTER(_dp), ctypes.c_int, _dp, _i64, _dp, _i64]
        _lib = L
    return _lib


def ref_lib():
    """The verbatim reference hsolve build, or None where it cannot be built."""
    global _ref
    if _ref is None:
        path = _build.REF_SO
        if not os.path.exists(path):
            try:
                path = _build.build_reference()
            except Exception:
                path = None
        if not path or not os.path.exists(path):
            return None
        R = ctypes.CDLL(path)
        R.ref_hsolve.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 _dp, _dp, _dp]
        _ref = R
    return _ref


def blas_lib():
    """libhsolve_blas.so bound to scipy's OpenBLAS (single-threaded BLAS), or
    None where that BLAS is absent."""
    global _blas
    if _blas is None:
        path = _build.BLAS_SO
        if not os.path.exists(path):
            _build.build_blas_port()
        blas = _build.scipy_openblas()
        if blas is None:
            return None
        B = ctypes.CDLL(path)
        B.hb_init.argtypes = [ctypes.c_char_p]
        B.hb_init.restype = ctypes.c_int
        if B.hb_init(blas.encode()) != 0:
            return None
        B.hb_hsolve.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                _dp, _dp, _dp]
        B.hb_hsolve.restype = ctypes.c_int
        B.hb_hsolve_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _i64, ctypes.POINTER(_dp),
                                   _i64, ctypes.c_int, _dp, _i64, ctypes.c_int]
        B.hb_hsolve_mt.restype = ctypes.c_int
        B.hb_matvec_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _i64, ctypes.POINTER(_dp),
                                   _i64, ctypes.POINTER(_dp), _i64, ctypes.POINTER(_dp), ctypes.c_int, _dp, _i64,
                                   _dp, _i64, ctypes.c_int]
        B.hb_copy_mt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _i64, ctypes.c_int]
        B.hb_fill_gaussian.argtypes = [_dp, _i64, _i64, _i64, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                       _i64, ctypes.c_int]
        _blas = B
    return _blas


def _p(a):
    assert a.dtype == np.float64
    return a.ctypes.data_as(_dp)


def _ld(a):
    """Leading dimension of a Fortran-ordered 2-D array (or a 1-D vector)."""
    if a.ndim == 1:
        return a.shape[0]
    assert a.strides[0] == 8, "expected column-major"
    return a.strides[1] // 8


# ---------------------------------------------------------------- generators

def seeds(master, n):
    out = (ctypes.c_long * n)()
    lib().orc_seeds(master, n, out)
    return np.array(out[:], dtype=np.int64)


def rand_matrix(seed_list, base, cols, offset=0):
    """Matrix(base, level, cols).rand() with the given per-block seeds."""
    nPart = len(seed_list)
    A = np.zeros((nPart * base, cols), order="F")
    s = (ctypes.c_long * nPart)(*[int(x) for x in seed_list])
    lib().orc_rand_matrix(s, nPart, base, cols, _p(A), offset)
    return A


def dense_blocks(useeds, vseeds, dseeds, m, rank, offset):
    nleaf = len(useeds)
    K = np.zeros((nleaf * m, m), order="F")
    mk = lambda v: (ctypes.c_long * nleaf)(*[int(x) for x in v])
    lib().orc_dense_blocks(mk(useeds), mk(vseeds), mk(dseeds), nleaf, m, rank, offset, _p(K), _ld(K))
    return K


# ---------------------------------------------------------------- LAPACK

def dgetrf(A):
    """LU with partial pivoting (netlib DGETRF).  Returns (LU, ipiv 1-based, info)."""
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    ipiv = np.zeros(min(m, n), dtype=np.int32)
    info = lib().orc_dgetrf(m, n, _p(A), _ld(A), ipiv.ctypes.data_as(_ip))
    return A, ipiv, info


def dgetrs(LU, ipiv, B, trans="N"):
    B = np.array(B, dtype=np.float64, order="F", copy=True)
    if B.ndim == 1:
        B = B.reshape(-1, 1, order="F")
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    LU = np.asfortranarray(LU)
    lib().orc_dgetrs(trans.encode(), LU.shape[0], B.shape[1], _p(LU), _ld(LU),
                     ipiv.ctypes.data_as(_ip), _p(B), _ld(B))
    return B


def dgemm(ta, tb, alpha, A, B, beta, C):
    A = np.asfortranarray(A)
    B = np.asfortranarray(B)
    C = np.array(C, dtype=np.float64, order="F", copy=True)
    m, n = C.shape
    k = A.shape[0] if ta in "tT" else A.shape[1]
    lib().orc_dgemm(ta.encode(), tb.encode(), m, n, k, alpha, _p(A), _ld(A), _p(B), _ld(B), beta, _p(C), _ld(C))
    return C


# ---------------------------------------------------------------- HODLR

def hsolve(nrow, nrhs, rank, nPart, K, U, V):
    """In-place restated hsolve (src/tasks/leaf_solve.cc:73-154)."""
    LD = _ld(K)
    assert _ld(U) == LD and _ld(V) == LD
    return lib().orc_hsolve(nrow, nrhs, rank, nPart, LD, _p(K), _p(U), _p(V))


def ref_hsolve(nrow, nrhs, rank, nPart, K, U, V):
    """In-place verbatim reference hsolve (None if it is not built here)."""
    R = ref_lib()
    if R is None:
        return None
    LD = _ld(K)
    assert _ld(U) == LD and _ld(V) == LD
    R.ref_hsolve(nrow, nrhs, rank, nPart, LD, _p(K), _p(U), _p(V))
    return 0


def _ptr_array(arrs):
    return (_dp * len(arrs))(*[_p(a) for a in arrs])


def hsolve_general(prob, B, keep_factors=False, nthreads=1):
    """Solve A X = B for a generalised HODLR problem (see problems.Problem).

    Returns (X, factors-dict or None, info).  The factors dict holds the leaf
    LU (N x m, stacked as the KTree region), leaf pivots, the transformed
    bases Utilde[l] (N x r each) and the capacitance LU / pivots by node.
    """
    L, m, r, N = prob.levels, prob.leaf, prob.rank, prob.n
    B = np.asarray(B, dtype=np.float64)
    if B.ndim == 1:
        B = B.reshape(-1, 1)
    k = B.shape[1]
    W = np.zeros((N, k + L * r), order="F")
    W[:, :k] = B
    for l in range(L):
        W[:, k + l * r:k + (l + 1) * r] = prob.U[l]
    K = np.array(prob.K, order="F", copy=True)
    Vs = [np.asfortranarray(v) for v in prob.V]
    Vp = _ptr_array(Vs)
    ss = [np.ascontiguousarray(s, dtype=np.float64) for s in prob.s] if prob.s is not None else None
    sp = _ptr_array(ss) if ss is not None else None
    ldv = _ld(Vs[0]) if L else N
    if nthreads > 1 and not keep_factors:
        info = lib().orc_hsolve_general_mt(m, L, r, _p(K), _ld(K), Vp, ldv, sp, k, _p(W), _ld(W), nthreads)
        return np.array(W[:, :k]), None, info
    nnode = (1 << L) - 1
    leaf_ipiv = np.zeros(N, dtype=np.int32)
    cap_lu = np.zeros(max(nnode, 1) * 4 * r * r)
    cap_ipiv = np.zeros(max(nnode, 1) * 2 * r, dtype=np.int32)
    info = lib().orc_hsolve_general(m, L, r, _p(K), _ld(K), Vp, ldv, sp, k, _p(W), _ld(W),
                                    leaf_ipiv.ctypes.data_as(_ip), _p(cap_lu), cap_ipiv.ctypes.data_as(_ip))
    X = np.array(W[:, :k])
    if not keep_factors:
        return X, None, info
    f = dict(leaf_lu=K, leaf_ipiv=leaf_ipiv.reshape(-1, m),
             utilde=[np.array(W[:, k + l * r:k + (l + 1) * r], order="F") for l in range(L)],
             cap_lu=cap_lu[:nnode * 4 * r * r].reshape(nnode, 2 * r, 2 * r).transpose(0, 2, 1),
             cap_ipiv=cap_ipiv[:nnode * 2 * r].reshape(nnode, 2 * r))
    return X, f, info


def hodlr_matvec(prob, X):
    """Y = A X in FP64 from the exact HODLR representation."""
    L, m, r = prob.levels, prob.leaf, prob.rank
    X = np.asfortranarray(np.asarray(X, dtype=np.float64).reshape(prob.n, -1))
    Y = np.zeros_like(X, order="F")
    Us = [np.asfortranarray(u) for u in prob.U]
    Vs = [np.asfortranarray(v) for v in prob.V]
    K = np.asfortranarray(prob.K)
    ld = _ld(Us[0]) if L else prob.n
    ss = [np.ascontiguousarray(s, dtype=np.float64) for s in prob.s] if prob.s is not None else None
    sp = _ptr_array(ss) if ss is not None else None
    lib().orc_hodlr_matvec(m, L, r, _p(K), _ld(K), _ptr_array(Us), ld, _ptr_array(Vs), ld, sp,
                           X.shape[1], _p(X), _ld(X), _p(Y), _ld(Y))
    return Y


# ---------------------------------------------------------------- irregular trees

def node_solve_irregular(r0, r1, VTu0, VTu1, VTd0, VTd1):
    """NodeSolveRegionTask::cpu_task (src/tasks/node_solve_region.cc:77-97)
    restated: S = I with S(i, r0+j) = VTu1(i, j), S(r0+j, i) = VTu0(j, i),
    B = [VTd1; VTd0], S.solve(B) (PtrMatrix::solve = dgesv,
    src/ptr_matrix.cc:101-111), the first r0 rows back into VTd1 and the last
    r1 into VTd0.  VTu0: r1 x r0, VTu1: r0 x r1, VTd0: r1 x k, VTd1: r0 x k.
    Returns (VTd0', VTd1', info)."""
    n = r0 + r1
    S = np.eye(n, order="F")
    for i in range(r0):
        for j in range(r1):
            S[i, r0 + j] = VTu1[i, j]
            S[r0 + j, i] = VTu0[j, i]
    B = np.asfortranarray(np.vstack([VTd1, VTd0]))
    LU, ipiv, info = dgetrf(S)
    X = dgetrs(LU, ipiv, B)
    return np.array(X[r0:], order="F"), np.array(X[:r0], order="F"), info


def tree_solve(tp, B):
    """Solve A X = B for an irregular tree (problems.TreeProblem) in the order
    of fastSolver2's SPMD solve (spmd_driver/solver_irregular_ranks.cc:145-235):
    every subtree solves its right-hand sides together with all of its
    top-level coupling columns (the hsolve of its own levels), then the top
    levels run deepest first -- VTu = V^T u and VTd = V^T d on each child
    (LMatrix::gemm), the node solve of unequal ranks (node_solve_irregular) and
    d -= u VTd (LMatrix::gemm_inplace), d being the solution columns and the
    coupling columns of the levels above."""
    T = tp.top_levels
    B = np.asarray(B, dtype=np.float64).reshape(tp.n, -1)
    k = B.shape[1]
    X = np.array(B, order="F")
    Ut = [np.zeros((tp.n, 64), order="F") for _ in range(T)]   # level l's transformed bases, child-wide ranks
    for (l, q, h), U in tp.Uc.items():
        rows = tp.child_rows(l, q, h)
        Ut[l][rows, :U.shape[1]] = U
    info = 0
    for j, sub in enumerate(tp.subs):
        rows = slice(tp.offsets[j], tp.offsets[j + 1])
        widths = [tp.u_rank(l, j) for l in range(T)]
        W = np.hstack([X[rows]] + [Ut[l][rows, :widths[l]] for l in range(T)])
        Xj, _, inf = hsolve_general(sub, W)
        info = info or inf
        X[rows] = Xj[:, :k]
        c = k
        for l in range(T):
            Ut[l][rows, :widths[l]] = Xj[:, c:c + widths[l]]
            c += widths[l]
    for l in range(T - 1, -1, -1):
        for q in range(1 << l):
            p = (1 << l) - 1 + q
            r0, r1 = tp.ranks[2 * p], tp.ranks[2 * p + 1]
            R = [tp.child_rows(l, q, h) for h in (0, 1)]
            j0 = [tp.child_leaves(l, q, h)[0] for h in (0, 1)]
            own = [Ut[l][R[0], :r0], Ut[l][R[1], :r1]]
            anc = [[(a, tp.u_rank(a, j0[h])) for a in range(l)] for h in (0, 1)]
            dcols = [np.hstack([X[R[h]]] + [Ut[a][R[h], :w] for a, w in anc[h]]) for h in (0, 1)]
            V = [tp.Vc[(l, q, 0)], tp.Vc[(l, q, 1)]]
            VTu0 = dgemm("T", "N", 1.0, V[0], own[0], 0.0, np.zeros((r1, r0)))
            VTu1 = dgemm("T", "N", 1.0, V[1], own[1], 0.0, np.zeros((r0, r1)))
            VTd0 = dgemm("T", "N", 1.0, V[0], dcols[0], 0.0, np.zeros((r1, dcols[0].shape[1])))
            VTd1 = dgemm("T", "N", 1.0, V[1], dcols[1], 0.0, np.zeros((r0, dcols[1].shape[1])))
            VTd0, VTd1, inf = node_solve_irregular(r0, r1, VTu0, VTu1, VTd0, VTd1)
            info = info or inf
            for h, eta in ((0, VTd1), (1, VTd0)):
                d = dgemm("N", "N", -1.0, own[h], eta, 1.0, dcols[h])
                X[R[h]] = d[:, :k]
                c = k
                for a, w in anc[h]:
                    Ut[a][R[h], :w] = d[:, c:c + w]
                    c += w
    return X, info


# ---------------------------------------------------------------- BLAS-backed restatement

def blas_hsolve(nrow, nrhs, rank, nPart, K, U, V):
    """In-place hsolve (src/tasks/leaf_solve.cc:73-154) with its dgemm_/dgesv_
    calls on scipy's OpenBLAS.  Returns INFO, or None without that BLAS."""
    B = blas_lib()
    if B is None:
        return None
    LD = _ld(K)
    assert _ld(U) == LD and _ld(V) == LD
    return B.hb_hsolve(nrow, nrhs, rank, nPart, LD, _p(K), _p(U), _p(V))


def blas_hsolve_mt(leaf, levels, rank, K, Vs, W, nrhs, nthreads):
    """In-place threaded hsolve with per-level V (hb_hsolve_mt): K (N x m
    stacked leaf blocks) becomes the leaf LU, W = [B | U^(0) | ...] becomes
    [X | Utilde^(0) | ...].  Returns 0, 1 (singular leaf) or 2 (singular
    capacitance system)."""
    B = blas_lib()
    assert B is not None, "scipy's OpenBLAS is not available"
    ldv = _ld(Vs[0]) if levels else K.shape[0]
    return B.hb_hsolve_mt(leaf, levels, rank, _p(K), _ld(K), _ptr_array(Vs), ldv, nrhs, _p(W), _ld(W), nthreads)


def blas_matvec(leaf, levels, rank, K, Us, Vs, ss, X, nthreads=None):
    """Y = A X in FP64 from the exact representation, threaded (hb_matvec_mt)."""
    B = blas_lib()
    assert B is not None, "scipy's OpenBLAS is not available"
    X = np.asfortranarray(X)
    Y = np.empty_like(X, order="F")
    ld = _ld(Us[0]) if levels else X.shape[0]
    sp = _ptr_array(ss) if ss is not None else None
    B.hb_matvec_mt(leaf, levels, rank, _p(K), _ld(K), _ptr_array(Us), ld, _ptr_array(Vs), ld, sp, X.shape[1],
                   _p(X), _ld(X), _p(Y), _ld(Y), nthreads or (os.cpu_count() or 1))
    return Y


def copy_mt(dst, src, nthreads=None):
    """dst[...] = src for two contiguous arrays of the same size, threaded."""
    assert dst.nbytes == src.nbytes
    B = blas_lib()
    if B is None:
        np.copyto(dst, src)
        return
    B.hb_copy_mt(dst.ctypes.data, src.ctypes.data, dst.nbytes, nthreads or (os.cpu_count() or 1))


def fill_gaussian(A, seed, scale=1.0, diag=0.0, diag_block=0, nthreads=None):
    """Fill the Fortran-ordered 2-D array A in place with seeded N(0, scale^2)
    values, plus `diag` on the diagonal of each diag_block x diag_block square
    of rows (the leaf blocks of a KTree region); threaded (hb_fill_gaussian)."""
    B = blas_lib()
    assert B is not None, "scipy's OpenBLAS is not available"
    B.hb_fill_gaussian(_p(A), A.shape[0], A.shape[1], _ld(A), seed, scale, diag, diag_block,
                       nthreads or (os.cpu_count() or 1))
