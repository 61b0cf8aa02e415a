"""GB300 HODLR fast direct solver -- Python bindings of the C ABI.

The product is ``libhodlr_gb300.so`` (CUDA, sm_103a) behind the C ABI in
``include/hodlr_gb300.h``.  This module loads it with ctypes and offers thin
wrappers that take torch CUDA tensors (torch is only the device-memory and
stream plumbing here).  There is no CPU fallback: every call goes to the
library, and loading fails loudly if the library is missing.
"""
import ctypes
import os
import struct

from . import build as _build

HODLR_OK = 0
HODLR_ERR_INVALID_ARG = 1
HODLR_ERR_CUDA = 2
HODLR_ERR_SINGULAR_LEAF = 3
HODLR_ERR_SINGULAR_CAPACITANCE = 4
HODLR_ERR_NOT_CONVERGED = 5
HODLR_ERR_NONFINITE_INPUT = 6
HODLR_ERR_TIMEOUT = 7
HODLR_ERR_NOT_FACTORED = 8
HODLR_ERR_OUT_OF_MEMORY = 9

FLAG_STREAM_INPUTS = 1

PREC_FP64 = 0
PREC_MIXED = 1
RESID_FP64 = 0
RESID_FP64_EMULATED = 1
RESID_FP64_TENSOR = 2

LIB_PATH = _build.LIB

PHASES = ["leaf_lu", "leaf_solve", "reduce", "capacitance", "update", "resid_leaf", "resid_reduce",
          "resid_update", "misc"]


class HodlrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("hodlr error %d: %s" % (code, msg))
        self.code = code


class Desc(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("leaf", ctypes.c_int32), ("levels", ctypes.c_int32),
                ("rank", ctypes.c_int32), ("nrhs_max", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("residual", ctypes.c_int32), ("refine_tol", ctypes.c_double),
                ("refine_max_iter", ctypes.c_int32), ("flags", ctypes.c_int32), ("stream", ctypes.c_void_p)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("status", ctypes.c_int32), ("bad_index", ctypes.c_int64),
                ("rel_residual", ctypes.c_double)]


class Grads(ctypes.Structure):
    _fields_ = [("db", ctypes.c_void_p), ("ldb", ctypes.c_int64), ("dD", ctypes.c_void_p),
                ("dU", ctypes.c_void_p), ("dV", ctypes.c_void_p), ("ds", ctypes.c_void_p)]


class Tuning(ctypes.Structure):
    _fields_ = [("red_ctas_per_sm", ctypes.c_int32), ("update_tile_rows", ctypes.c_int32),
                ("cap_warps", ctypes.c_int32), ("update_tc_shape", ctypes.c_int32), ("leaf_apply", ctypes.c_int32),
                ("ms", ctypes.c_double)]

    def as_dict(self):
        return {"red_ctas_per_sm": self.red_ctas_per_sm, "update_tile_rows": self.update_tile_rows,
                "cap_warps": self.cap_warps, "update_tc_shape": self.update_tc_shape, "leaf_apply": self.leaf_apply,
                "ms": self.ms}


class System(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("leaf", ctypes.c_int32), ("levels", ctypes.c_int32),
                ("rank", ctypes.c_int32), ("nrhs", ctypes.c_int32)]


class TreeDesc(ctypes.Structure):
    _fields_ = [("top_levels", ctypes.c_int32), ("subtrees", ctypes.POINTER(Desc)),
                ("coupling_rank", ctypes.POINTER(ctypes.c_int32)), ("nrhs_max", ctypes.c_int32),
                ("flags", ctypes.c_int32), ("stream", ctypes.c_void_p)]


class BatchDesc(ctypes.Structure):
    _fields_ = [("systems", ctypes.POINTER(System)), ("count", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("residual", ctypes.c_int32), ("refine_tol", ctypes.c_double), ("refine_max_iter", ctypes.c_int32),
                ("flags", ctypes.c_int32), ("stream", ctypes.c_void_p)]


# name -> (restype, argtypes); the full exported surface of include/hodlr_gb300.h
_VP, _I, _I64, _D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
SIGNATURES = {
    "hodlr_hsolve": (_I, [_I, _I, _I, _I, _I, _VP, _VP, _VP]),
    "hodlr_hsolve_ex": (_I, [_I, _I, _I, _I, _I, _VP, _VP, _VP, _I, _VP, ctypes.POINTER(SolveInfo)]),
    "hodlr_create": (_I, [ctypes.POINTER(Desc), ctypes.POINTER(_VP)]),
    "hodlr_destroy": (_I, [_VP]),
    "hodlr_set_stream": (_I, [_VP, _VP]),
    "hodlr_set_leaf_blocks": (_I, [_VP, _VP, _I64, _I64]),
    "hodlr_set_lowrank": (_I, [_VP, _I, _VP, _I64, _VP, _I64, _VP]),
    "hodlr_factor": (_I, [_VP]),
    "hodlr_solve": (_I, [_VP, _VP, _I64, _I, ctypes.POINTER(SolveInfo)]),
    "hodlr_solve_transpose": (_I, [_VP, _VP, _I64, _I, ctypes.POINTER(SolveInfo)]),
    "hodlr_matvec": (_I, [_VP, _I, _VP, _I64, _VP, _I64, _I]),
    "hodlr_adjoint": (_I, [_VP, _VP, _I64, _VP, _I64, _I, ctypes.POINTER(Grads)]),
    "hodlr_get_factors": (_I, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "hodlr_get_inputs": (_I, [_VP, _VP, _I64, _I64, _VP, _VP, _VP]),
    "hodlr_pad_rows": (_I, [_I, _VP, _I, _I, _VP, _I64, _VP, _I64, _VP]),
    "hodlr_unpad_rows": (_I, [_I, _VP, _I, _I, _VP, _I64, _VP, _I64, _VP]),
    "hodlr_pad_leaf_blocks": (_I, [_I, _VP, _I, _VP, _VP, _VP]),
    "hodlr_draw_seeds": (_I, [_I64, _I, _VP]),
    "hodlr_rand_matrix": (_I, [_VP, _I, _I64, _I, _D, _VP, _I64, _VP]),
    "hodlr_set_seeded": (_I, [_VP, _VP, _VP, _VP, _D]),
    "hodlr_checkpoint_size": (_I, [_VP, ctypes.POINTER(_I64)]),
    "hodlr_checkpoint_save": (_I, [_VP, _VP, _I64]),
    "hodlr_checkpoint_load": (_I, [_VP, _I64, _VP, ctypes.POINTER(_VP)]),
    "hodlr_set_uvd": (_I, [_VP, _VP, _I64, _VP, _I64, _VP]),
    "hodlr_gemm_reduce": (_I, [_I, _I, _I, _I, _VP, _I64, _VP, _I64, _VP, _I64]),
    "hodlr_gemm_reduce_noalloc": (_I, [_I, _I, _I, _I, _VP, _I64, _VP, _I64, _VP, _I64]),
    "hodlr_debug_wait_fault": (_I, [_I, _I, _I64]),
    "hodlr_gemm_broadcast": (_I, [_I, _I, _I, _I, _I, _D, _VP, _I64, _VP, _I64, _D, _VP, _I64]),
    "hodlr_node_solve": (_I, [_I, _I, _I, _VP, _I64, _VP, _I64]),
    "hodlr_node_solve_irregular": (_I, [_I, _I, _I, _I, _VP, _I64, _VP, _I64, _VP, _I64, _VP, _I64]),
    "hodlr_tree_create": (_I, [ctypes.POINTER(TreeDesc), ctypes.POINTER(_VP)]),
    "hodlr_tree_destroy": (_I, [_VP]),
    "hodlr_tree_subtree": (_I, [_VP, _I, ctypes.POINTER(_VP)]),
    "hodlr_tree_rows": (_I, [_VP, ctypes.POINTER(_I64), _VP]),
    "hodlr_tree_set_coupling": (_I, [_VP, _I, _I, _I, _VP, _I64, _VP, _I64]),
    "hodlr_tree_factor": (_I, [_VP]),
    "hodlr_tree_solve": (_I, [_VP, _VP, _I64, _I, ctypes.POINTER(SolveInfo)]),
    "hodlr_tree_matvec": (_I, [_VP, _VP, _I64, _VP, _I64, _I]),
    "hodlr_generate": (_I, [_VP, ctypes.c_uint64, _D, _I, _D, _VP, _I64, _I]),
    "hodlr_profile": (_I, [_VP, _I, _VP, _VP, _I]),
    "hodlr_last_timings": (_I, [_VP, ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    "hodlr_batch_create": (_I, [ctypes.POINTER(BatchDesc), ctypes.POINTER(_VP)]),
    "hodlr_batch_destroy": (_I, [_VP]),
    "hodlr_batch_set_leaf_blocks": (_I, [_VP, _I, _VP, _I64, _I64]),
    "hodlr_batch_set_lowrank": (_I, [_VP, _I, _I, _VP, _I64, _VP, _I64, _VP]),
    "hodlr_batch_generate": (_I, [_VP, ctypes.c_uint64, _D, _VP, _VP]),
    "hodlr_batch_factor": (_I, [_VP]),
    "hodlr_batch_solve": (_I, [_VP, _VP, _VP, ctypes.POINTER(SolveInfo)]),
    "hodlr_batch_stats": (_I, [_VP, ctypes.POINTER(_I), ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    "hodlr_autotune": (_I, [_VP, _I, ctypes.POINTER(Tuning)]),
    "hodlr_set_tuning": (_I, [_VP, ctypes.POINTER(Tuning)]),
    "hodlr_get_tuning": (_I, [_VP, ctypes.POINTER(Tuning)]),
    "hodlr_batch_autotune": (_I, [_VP, ctypes.POINTER(Tuning), _I]),
    "hodlr_kernel_launches": (_I64, []),
    "hodlr_last_error_string": (ctypes.c_char_p, []),
}

_lib = None


def lib(build_if_missing=False):
    """Load libhodlr_gb300.so.  Raises if it is absent (no fallback path)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise ImportError("libhodlr_gb300.so is not built (run __graft_entry__.build() "
                                  "or python fastsolver2_gb300/build.py)")
            _build.build()
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code):
    if code != HODLR_OK:
        raise HodlrError(code, lib().hodlr_last_error_string().decode())
    return code


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _ld(t):
    """Leading dimension of a column-major (Fortran-ordered) 2-D tensor."""
    if t.dim() == 1 or t.shape[1] == 1:
        assert t.dim() == 1 or t.stride(0) == 1 or t.shape[0] == 1, "expected a column-major tensor"
        return t.shape[0]
    assert t.stride(0) == 1, "expected a column-major tensor (use .t().contiguous().t())"
    return t.stride(1)


def colmajor(t):
    """A column-major copy of a 2-D tensor (torch is row-major by default)."""
    return t.t().contiguous().t()


class Solver:
    """Handle-based factor/solve API (hodlr_create ... hodlr_destroy).

    Without ``stream`` the library works on a non-blocking stream of its own:
    tensors that torch kernels have just written must be finished
    (``torch.cuda.synchronize()``) before they are passed in.  Every call that
    returns results (factor, solve, matvec, adjoint, get_*) has finished its
    device work when it returns."""

    def __init__(self, n, leaf, levels, rank, nrhs_max=1, precision=PREC_FP64, residual=RESID_FP64_TENSOR,
                 refine_tol=1e-12, refine_max_iter=10, stream=None, flags=0):
        self.h = None
        self.desc = Desc(n, leaf, levels, rank, nrhs_max, precision, residual, refine_tol, refine_max_iter, flags,
                         stream)
        h = ctypes.c_void_p()
        check(lib().hodlr_create(ctypes.byref(self.desc), ctypes.byref(h)))
        self.h = h
        self.n, self.leaf, self.levels, self.rank = n, leaf, levels, rank

    def close(self):
        if self.h:
            lib().hodlr_destroy(self.h)
            self.h = None

    __del__ = close

    def set_leaf_blocks(self, D, ld=None, leaf_stride=None):
        """D: torch float64 CUDA tensor; default layout = the KTree region (N x m column-major)."""
        ld = _ld(D) if ld is None else ld
        stride = self.leaf if leaf_stride is None else leaf_stride
        check(lib().hodlr_set_leaf_blocks(self.h, _ptr(D), ld, stride))

    def set_lowrank(self, level, U, V, s=None):
        check(lib().hodlr_set_lowrank(self.h, level, _ptr(U), _ld(U), _ptr(V), _ld(V), _ptr(s)))

    def factor(self):
        check(lib().hodlr_factor(self.h))

    def solve(self, B, transpose=False):
        info = SolveInfo()
        f = lib().hodlr_solve_transpose if transpose else lib().hodlr_solve
        check(f(self.h, _ptr(B), _ld(B), B.shape[1] if B.dim() == 2 else 1, ctypes.byref(info)))
        return info

    def matvec(self, X, Y, transpose=False):
        check(lib().hodlr_matvec(self.h, int(transpose), _ptr(X), _ld(X), _ptr(Y), _ld(Y),
                                 X.shape[1] if X.dim() == 2 else 1))

    def adjoint(self, x, g, db=None, dD=None, dU=None, dV=None, ds=None):
        gr = Grads(_ptr(db), _ld(db) if db is not None else 0, _ptr(dD), _ptr(dU), _ptr(dV), _ptr(ds))
        check(lib().hodlr_adjoint(self.h, _ptr(x), _ld(x), _ptr(g), _ld(g),
                                  x.shape[1] if x.dim() == 2 else 1, ctypes.byref(gr)))

    def get_factors(self, leaf_lu=None, leaf_ipiv=None, utilde=None, cap_lu=None, cap_ipiv=None):
        check(lib().hodlr_get_factors(self.h, _ptr(leaf_lu), _ptr(leaf_ipiv), _ptr(utilde), _ptr(cap_lu),
                                      _ptr(cap_ipiv)))

    def generate(self, seed, shift=4.0, orthonormal=False, decay=0.0, B=None):
        check(lib().hodlr_generate(self.h, seed, shift, int(orthonormal), decay, _ptr(B),
                                   _ld(B) if B is not None else 0, B.shape[1] if B is not None else 0))

    def get_inputs(self, D=None, ld=None, leaf_stride=None, U=None, V=None, s=None):
        """Copy the problem out (torch tensors, host or device)."""
        ld = self.leaf if ld is None else ld
        stride = self.leaf * self.leaf if leaf_stride is None else leaf_stride
        check(lib().hodlr_get_inputs(self.h, _ptr(D), ld, stride, _ptr(U), _ptr(V), _ptr(s)))

    def set_seeded(self, useeds, vseeds, dseeds, offset=0.0):
        """Inputs from per-leaf drand48 seeds, as the reference's HMatrix::init builds them."""
        a = [_seed_array(x) for x in (useeds, vseeds, dseeds)]
        check(lib().hodlr_set_seeded(self.h, a[0], a[1], a[2], float(offset)))

    def checkpoint(self):
        """The factored state as bytes (hodlr_checkpoint_save)."""
        nb = _I64()
        check(lib().hodlr_checkpoint_size(self.h, ctypes.byref(nb)))
        buf = ctypes.create_string_buffer(nb.value)
        check(lib().hodlr_checkpoint_save(self.h, buf, nb.value))
        return buf.raw

    @classmethod
    def from_checkpoint(cls, data, stream=None):
        """A factored Solver from bytes written by checkpoint() (hodlr_checkpoint_load)."""
        h = ctypes.c_void_p()
        check(lib().hodlr_checkpoint_load(data, len(data), stream, ctypes.byref(h)))
        self = cls.__new__(cls)
        self.h = h
        self.desc = None
        # header: magic[8], version, nbuf (uint32), n (int64), leaf, levels, rank (int32)
        self.n, self.leaf, self.levels, self.rank = struct.unpack_from("<q3i", data, 16)
        return self

    def profile(self, enable=-1, read=False):
        """Switch per-phase timing on/off; with read=True return {phase: (ms, launches)} and reset."""
        if not read:
            check(lib().hodlr_profile(self.h, enable, None, None, 0))
            return None
        ms = (ctypes.c_double * len(PHASES))()
        n = (ctypes.c_int64 * len(PHASES))()
        check(lib().hodlr_profile(self.h, enable, ms, n, len(PHASES)))
        return {name: (ms[i], n[i]) for i, name in enumerate(PHASES)}

    def autotune(self, nrhs=1):
        """Pick the launch shapes by timing factor + solve; leaves the handle factored."""
        t = Tuning()
        check(lib().hodlr_autotune(self.h, nrhs, ctypes.byref(t)))
        return t.as_dict()

    def set_tuning(self, red_ctas_per_sm=4, update_tile_rows=0, cap_warps=0, update_tc_shape=0, leaf_apply=0):
        t = Tuning(red_ctas_per_sm, update_tile_rows, cap_warps, update_tc_shape, leaf_apply, -1.0)
        check(lib().hodlr_set_tuning(self.h, ctypes.byref(t)))

    def get_tuning(self):
        t = Tuning()
        check(lib().hodlr_get_tuning(self.h, ctypes.byref(t)))
        return t.as_dict()

    def timings(self):
        f, s = ctypes.c_double(), ctypes.c_double()
        check(lib().hodlr_last_timings(self.h, ctypes.byref(f), ctypes.byref(s)))
        return f.value, s.value


class Batch:
    """Ragged batch of independent systems (hodlr_batch_*).

    systems: list of (n, leaf, levels, rank, nrhs).  Right-hand sides are
    column-major float64 CUDA tensors, one per system.  As for Solver, torch
    work that produced an input must be finished before it is passed in."""

    def __init__(self, systems, precision=PREC_FP64, residual=RESID_FP64_TENSOR, refine_tol=1e-12,
                 refine_max_iter=10, stream=None):
        self.h = None
        self.systems = [tuple(int(v) for v in s) for s in systems]
        arr = (System * len(self.systems))(*[System(*s) for s in self.systems])
        self._arr = arr
        self.desc = BatchDesc(arr, len(self.systems), precision, residual, refine_tol, refine_max_iter, 0, stream)
        h = ctypes.c_void_p()
        check(lib().hodlr_batch_create(ctypes.byref(self.desc), ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().hodlr_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def __len__(self):
        return len(self.systems)

    @staticmethod
    def _ptrs(Bs):
        n = len(Bs)
        ptrs = (ctypes.c_void_p * n)(*[b.data_ptr() if b is not None else None for b in Bs])
        lds = (ctypes.c_int64 * n)(*[_ld(b) if b is not None else 0 for b in Bs])
        return ptrs, lds

    def set_leaf_blocks(self, i, D, ld=None, leaf_stride=None):
        leaf = self.systems[i][1]
        ld = _ld(D) if ld is None else ld
        stride = leaf if leaf_stride is None else leaf_stride
        check(lib().hodlr_batch_set_leaf_blocks(self.h, i, _ptr(D), ld, stride))

    def set_lowrank(self, i, level, U, V, s=None):
        check(lib().hodlr_batch_set_lowrank(self.h, i, level, _ptr(U), _ld(U), _ptr(V), _ld(V), _ptr(s)))

    def generate(self, seed, shift=4.0, Bs=None):
        if Bs is None:
            check(lib().hodlr_batch_generate(self.h, seed, shift, None, None))
        else:
            ptrs, lds = self._ptrs(Bs)
            check(lib().hodlr_batch_generate(self.h, seed, shift, ptrs, lds))

    def factor(self):
        check(lib().hodlr_batch_factor(self.h))

    def solve(self, Bs):
        """Solve in place; returns the per-system SolveInfo list."""
        ptrs, lds = self._ptrs(Bs)
        info = (SolveInfo * len(Bs))()
        check(lib().hodlr_batch_solve(self.h, ptrs, lds, info))
        return list(info)

    def autotune(self):
        """Per-forest launch shapes by timing; the batch must be factored again."""
        nf = self.stats()[0]
        arr = (Tuning * max(nf, 1))()
        check(lib().hodlr_batch_autotune(self.h, arr, nf))
        return [arr[i].as_dict() for i in range(nf)]

    def stats(self):
        nf, f, s = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        check(lib().hodlr_batch_stats(self.h, ctypes.byref(nf), ctypes.byref(f), ctypes.byref(s)))
        return nf.value, f.value, s.value


class _Subtree(Solver):
    """A tree's subtree handle (owned by the tree: close() does not destroy it)."""

    def __init__(self, h, n, leaf, levels, rank):
        self.h, self.desc = h, None
        self.n, self.leaf, self.levels, self.rank = n, leaf, levels, rank

    def close(self):
        self.h = None

    __del__ = close


class Tree:
    """Irregular tree (hodlr_tree_*): 2^T uniform subtrees, each with its own
    leaf size, depth, rank and precision, under T top levels whose nodes couple
    their children with ranks (r0, r1) that may differ.

    subtrees: list of (leaf, levels, rank) or dicts with those keys and
    optionally precision / residual / refine_tol / refine_max_iter.
    coupling_ranks: 2 (2^T - 1) ranks, node p = 2^l - 1 + q first child then
    second.  Each subtree is a Solver-like handle (``tree.subtree(j)``) whose
    set_* calls fill its leaves and bases."""

    def __init__(self, top_levels, subtrees, coupling_ranks, nrhs_max=1, precision=PREC_FP64,
                 residual=RESID_FP64_TENSOR, refine_tol=1e-12, refine_max_iter=10, stream=None):
        self.h = None
        nsub = 1 << top_levels
        if len(subtrees) != nsub or len(coupling_ranks) != 2 * (nsub - 1):
            raise ValueError("need 2^T subtrees and 2 (2^T - 1) coupling ranks")
        descs = (Desc * nsub)()
        self._shapes = []
        for j, sd in enumerate(subtrees):
            if not isinstance(sd, dict):
                sd = dict(zip(("leaf", "levels", "rank"), sd))
            leaf, levels, rank = sd["leaf"], sd["levels"], sd["rank"]
            descs[j] = Desc(leaf << levels, leaf, levels, rank, 1, sd.get("precision", precision),
                            sd.get("residual", residual), sd.get("refine_tol", refine_tol),
                            sd.get("refine_max_iter", refine_max_iter), 0, None)
            self._shapes.append((leaf << levels, leaf, levels, rank))
        ranks = (ctypes.c_int32 * len(coupling_ranks))(*[int(r) for r in coupling_ranks])
        self.desc = TreeDesc(top_levels, descs, ranks, nrhs_max, 0, stream)
        self._keep = (descs, ranks)
        h = ctypes.c_void_p()
        check(lib().hodlr_tree_create(ctypes.byref(self.desc), ctypes.byref(h)))
        self.h = h
        self.top_levels, self.ranks = top_levels, list(coupling_ranks)
        n = _I64()
        offs = (_I64 * (nsub + 1))()
        check(lib().hodlr_tree_rows(self.h, ctypes.byref(n), offs))
        self.n, self.offsets = n.value, [offs[i] for i in range(nsub + 1)]

    def close(self):
        if self.h:
            lib().hodlr_tree_destroy(self.h)
            self.h = None

    __del__ = close

    def subtree(self, j):
        h = ctypes.c_void_p()
        check(lib().hodlr_tree_subtree(self.h, j, ctypes.byref(h)))
        return _Subtree(h, *self._shapes[j])

    def set_coupling(self, level, pos, child, U, V):
        check(lib().hodlr_tree_set_coupling(self.h, level, pos, child, _ptr(U), _ld(U), _ptr(V), _ld(V)))

    def factor(self):
        check(lib().hodlr_tree_factor(self.h))

    def solve(self, B):
        info = SolveInfo()
        check(lib().hodlr_tree_solve(self.h, _ptr(B), _ld(B), B.shape[1] if B.dim() == 2 else 1,
                                     ctypes.byref(info)))
        return info

    def matvec(self, X, Y):
        check(lib().hodlr_tree_matvec(self.h, _ptr(X), _ld(X), _ptr(Y), _ld(Y), X.shape[1] if X.dim() == 2 else 1))


def node_solve_irregular(nnode, r0, r1, VTu0, VTu1, VTd0, VTd1):
    """NodeSolveRegionTask for nnode stacked nodes (hodlr_node_solve_irregular), in place on VTd0 / VTd1."""
    nrhs = VTd0.shape[1] if VTd0.dim() == 2 else 1
    check(lib().hodlr_node_solve_irregular(nnode, r0, r1, nrhs, _ptr(VTu0), _ld(VTu0), _ptr(VTu1), _ld(VTu1),
                                           _ptr(VTd0), _ld(VTd0), _ptr(VTd1), _ld(VTd1)))


def hsolve(nrow, nrhs, rank, nPart, LD, K, U, V, precision=PREC_FP64, stream=None):
    """fastSolver2's hsolve(nrow, nrhs, rank, nPart, LD, K, U, V), in place.

    K, U, V: torch float64 tensors (CUDA, column-major, leading dimension LD)
    or numpy Fortran-ordered float64 arrays (host; staged by the library)."""
    def p(a):
        if a is None:
            return None
        if hasattr(a, "data_ptr"):
            return ctypes.c_void_p(a.data_ptr())
        return ctypes.c_void_p(a.ctypes.data)
    info = SolveInfo()
    check(lib().hodlr_hsolve_ex(nrow, nrhs, rank, nPart, LD, p(K), p(U), p(V), precision, stream,
                                ctypes.byref(info)))
    return info


def _seed_array(seeds):
    seeds = [int(x) for x in seeds]
    return (ctypes.c_int64 * max(1, len(seeds)))(*seeds)


def _sizes(sz):
    sz = [int(x) for x in sz]
    return (ctypes.c_int32 * max(1, len(sz)))(*sz), len(sz)


def pad_rows(sizes, m_max, src, dst, stream=None):
    """Rows of leaf i of src (packed, CUDA float64 column-major) to rows i*m_max.. of dst, zero padding."""
    a, n = _sizes(sizes)
    cols = src.shape[1] if src.dim() == 2 else 1
    check(lib().hodlr_pad_rows(n, a, int(m_max), cols, _ptr(src), _ld(src), _ptr(dst), _ld(dst), stream))


def unpad_rows(sizes, m_max, src, dst, stream=None):
    """The inverse of pad_rows: padded src to packed dst."""
    a, n = _sizes(sizes)
    cols = src.shape[1] if src.dim() == 2 else 1
    check(lib().hodlr_unpad_rows(n, a, int(m_max), cols, _ptr(src), _ld(src), _ptr(dst), _ld(dst), stream))


def pad_leaf_blocks(sizes, m_max, src, dst, stream=None):
    """Leaf blocks packed one after another (sz_i x sz_i, column-major) to [nleaf][m_max][m_max]."""
    a, n = _sizes(sizes)
    check(lib().hodlr_pad_leaf_blocks(n, a, int(m_max), _ptr(src), _ptr(dst), stream))


def draw_seeds(master, n):
    """Matrix::rand's per-partition seeds: srand48(master), n lrand48 draws."""
    out = (ctypes.c_int64 * max(1, n))()
    check(lib().hodlr_draw_seeds(int(master), int(n), out))
    return [out[i] for i in range(n)]


def rand_matrix(seeds, rows, A, offset=0.0, stream=None):
    """Fill A (CUDA float64, column-major) with len(seeds) row partitions of `rows` rows, each from its
    seed's drand48 stream in row-major order (the reference's PtrMatrix::rand)."""
    cols = A.shape[1] if A.dim() == 2 else 1
    check(lib().hodlr_rand_matrix(_seed_array(seeds), len(seeds), rows, cols, float(offset), _ptr(A), _ld(A),
                                  stream))


def debug_wait_fault(cta=-1, stage=0, budget_cycles=0):
    """Test hook of the bounded device waits (see hodlr_debug_wait_fault);
    cta=-1 switches it off."""
    check(lib().hodlr_debug_wait_fault(cta, stage, budget_cycles))


def kernel_launches():
    return lib().hodlr_kernel_launches()
