"""Irregular trees without padding (hodlr_tree_*, hodlr_node_solve_irregular):
uniform subtrees with their own leaf size, depth and rank under top levels
whose nodes couple their children with unequal ranks, as fastSolver2's SPMD
drivers build them (spmd_driver/solver_irregular_part.cc:73-79, ten times the
leaf size on the first `-heavy` shards; solver_irregular_ranks.cc:99-132,
rank0 / rank1 shards coupled with the sibling's rank).

* the (r0+r1)-square node solve against the oracle's restatement of
  NodeSolveRegionTask (src/tasks/node_solve_region.cc:77-97): 1e-13 relative;
* tree solves against a dense FP64 solve and against the oracle's tree solve
  in the SPMD driver's order: 1e-11 relative (FP64 subtrees), 1e-10 (mixed
  subtrees refined to 1e-12);
* the heavy-leaf case of solver_irregular_part.cc (one subtree of four with
  leaf 640, the others leaf 64): the native tree against the same matrix
  embedded in the uniform tree with every leaf padded to 640, same solution,
  a third of the rows and less time.
"""
import time

import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle import problems as P
from tests.test_gpu_solver import rel, to_dev, to_host

pytestmark = pytest.mark.gpu


def make_tree(fs, tp, nrhs, precision=0, **kw):
    shapes = [(s.leaf, s.levels, s.rank) for s in tp.subs]
    t = fs.Tree(tp.top_levels, shapes, tp.ranks, nrhs_max=nrhs, precision=precision, **kw)
    keep = []
    for j, s in enumerate(tp.subs):
        st = t.subtree(j)
        D = to_dev(s.K)
        keep.append(D)
        st.set_leaf_blocks(D)
        for l in range(s.levels):
            U, V = to_dev(s.U[l]), to_dev(s.V[l])
            sv = to_dev(s.s[l]) if s.s is not None else None
            keep += [U, V, sv]
            st.set_lowrank(l, U, V, sv)
    for (l, q, h), U in tp.Uc.items():
        Ud, Vd = to_dev(U), to_dev(tp.Vc[(l, q, h)])
        keep += [Ud, Vd]
        t.set_coupling(l, q, h, Ud, Vd)
    torch.cuda.synchronize()
    t.inputs = keep
    return t


@pytest.mark.parametrize("nnode,r0,r1,nrhs", [(1, 12, 5, 3), (3, 3, 16, 1), (2, 64, 64, 40), (4, 1, 64, 33)])
def test_node_solve_irregular_matches_oracle(hodlr, nnode, r0, r1, nrhs):
    rng = np.random.default_rng(nnode * 100 + r0 + r1)
    VTu0 = rng.standard_normal((nnode * r1, r0)) * (0.4 / np.sqrt(r0 + r1))
    VTu1 = rng.standard_normal((nnode * r0, r1)) * (0.4 / np.sqrt(r0 + r1))
    VTd0 = rng.standard_normal((nnode * r1, nrhs))
    VTd1 = rng.standard_normal((nnode * r0, nrhs))
    d0, d1 = to_dev(VTd0), to_dev(VTd1)
    hodlr.node_solve_irregular(nnode, r0, r1, to_dev(VTu0), to_dev(VTu1), d0, d1)
    g0, g1 = to_host(d0), to_host(d1)
    for p in range(nnode):
        s0, s1 = slice(p * r1, (p + 1) * r1), slice(p * r0, (p + 1) * r0)
        o0, o1, info = O.node_solve_irregular(r0, r1, VTu0[s0], VTu1[s1], VTd0[s0], VTd1[s1])
        assert info == 0
        scale = max(np.linalg.norm(o0), np.linalg.norm(o1))
        assert np.linalg.norm(g0[s0] - o0) <= 1e-13 * scale
        assert np.linalg.norm(g1[s1] - o1) <= 1e-13 * scale


def test_node_solve_irregular_reports_singular_system(hodlr):
    r0, r1 = 3, 2
    VTu0 = np.zeros((r1, r0))
    VTu1 = np.zeros((r0, r1))
    VTu1[0, 0] = VTu0[0, 0] = 1.0     # rows 0 and r0 of S equal: S singular
    with pytest.raises(hodlr.HodlrError) as e:
        hodlr.node_solve_irregular(1, r0, r1, to_dev(VTu0), to_dev(VTu1), to_dev(np.ones((r1, 1))),
                                   to_dev(np.ones((r0, 1))))
    assert e.value.code == hodlr.HODLR_ERR_SINGULAR_CAPACITANCE


TREES = {
    # solver_irregular_part.cc: one heavy shard (leaf x10) of two
    "heavy2": (1, [(32, 3, 4), (320, 3, 4)], [4, 4]),
    # solver_irregular_ranks.cc: shard ranks rank0 / rank1 coupled with the sibling's rank
    "ranks2": (1, [(64, 3, 12), (64, 3, 5)], [12, 5]),
    # both at once, two top levels, every node with its own pair of ranks
    "mixed4": (2, [(320, 2, 8), (32, 2, 8), (32, 3, 5), (64, 2, 3)], [7, 12, 5, 9, 16, 2]),
    # three top levels: ancestors of unequal ranks above the nodes of one depth
    "deep8": (3, [(16, 1, 2)] * 3 + [(48, 1, 3)] * 5, list(range(1, 15))),
}


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", sorted(TREES))
def test_tree_solve_matches_dense_and_oracle(hodlr, name, precision):
    T, shapes, ranks = TREES[name]
    tp = P.tree_problem(T, shapes, ranks, nrhs=5, seed=len(name) + T)
    t = make_tree(hodlr, tp, nrhs=5, precision=precision, refine_tol=1e-12)
    assert t.n == tp.n and t.offsets == tp.offsets
    t.factor()
    Bd = to_dev(tp.B)
    info = t.solve(Bd)
    X = to_host(Bd)
    Xd = np.linalg.solve(tp.dense(), tp.B)
    Xo, oinfo = O.tree_solve(tp, tp.B)
    assert oinfo == 0 and rel(Xo, Xd) < 1e-13
    tol = 1e-11 if precision == 0 else 1e-10
    assert rel(X, Xd) < tol and rel(X, Xo) < tol
    if precision == 1:
        assert 0.0 <= info.rel_residual <= 1e-12 and info.iterations >= 1
    # a second solve with fewer columns reuses the factorisation
    B2 = to_dev(tp.B[:, :2])
    t.solve(B2)
    assert rel(to_host(B2), Xd[:, :2]) < tol
    t.close()


def test_tree_matvec_matches_dense(hodlr):
    T, shapes, ranks = TREES["mixed4"]
    tp = P.tree_problem(T, shapes, ranks, nrhs=3, seed=9)
    t = make_tree(hodlr, tp, nrhs=3)
    Xh = np.asfortranarray(np.random.default_rng(2).standard_normal((tp.n, 3)))
    Y = torch.empty((3, tp.n), dtype=torch.float64, device="cuda").t()
    t.matvec(to_dev(Xh), Y)
    ref = tp.dense() @ Xh
    assert rel(to_host(Y), ref) < 1e-14
    t.close()


def test_tree_rejects_unset_coupling_and_bad_ranks(hodlr):
    with pytest.raises(hodlr.HodlrError):
        hodlr.Tree(1, [(32, 2, 4), (32, 2, 4)], [65, 4])
    tp = P.tree_problem(1, [(32, 2, 4), (32, 2, 4)], [3, 6], nrhs=1, seed=1)
    t = hodlr.Tree(1, [(32, 2, 4), (32, 2, 4)], [3, 6])
    with pytest.raises(hodlr.HodlrError) as e:
        t.factor()
    assert e.value.code == hodlr.HODLR_ERR_NOT_FACTORED
    t.close()


def _padded_uniform(hodlr, tp, m_max, nrhs):
    """The same matrix in the uniform tree with every leaf padded to m_max
    (identity blocks, zero rows of U, V and B)."""
    T, subs = tp.top_levels, tp.subs
    Ls = subs[0].levels
    assert all(s.levels == Ls for s in subs) and len(set(tp.ranks)) == 1
    r = tp.ranks[0]
    assert all(s.rank == r for s in subs)
    sizes = np.concatenate([[s.leaf] * (1 << s.levels) for s in subs])
    nleaf, n_pad = len(sizes), len(sizes) * m_max
    packed = np.concatenate([s.leaf_block(i).ravel(order="F") for s in subs for i in range(1 << s.levels)])
    Dp = torch.empty(nleaf * m_max * m_max, dtype=torch.float64, device="cuda")
    hodlr.pad_leaf_blocks(sizes, m_max, torch.from_numpy(packed).cuda(), Dp)
    s = hodlr.Solver(n_pad, m_max, T + Ls, r, nrhs_max=nrhs)
    s.set_leaf_blocks(Dp, ld=m_max, leaf_stride=m_max * m_max)
    keep = [Dp]
    for l in range(T + Ls):
        U, V = np.zeros((tp.n, r), order="F"), np.zeros((tp.n, r), order="F")
        if l < T:
            for (ll, q, h), Uc in tp.Uc.items():
                if ll == l:
                    rows = tp.child_rows(l, q, h)
                    U[rows], V[rows] = Uc, tp.Vc[(l, q, h)]
        else:
            for j, sub in enumerate(subs):
                rows = slice(tp.offsets[j], tp.offsets[j + 1])
                U[rows], V[rows] = sub.U[l - T], sub.V[l - T]
        Up = torch.empty((r, n_pad), dtype=torch.float64, device="cuda").t()
        Vp = torch.empty((r, n_pad), dtype=torch.float64, device="cuda").t()
        hodlr.pad_rows(sizes, m_max, to_dev(U), Up)
        hodlr.pad_rows(sizes, m_max, to_dev(V), Vp)
        keep += [Up, Vp]
        s.set_lowrank(l, Up, Vp)
    torch.cuda.synchronize()
    s.inputs = keep
    return s, sizes, n_pad


def _best_seconds(fn, reps=3):
    best = float("inf")
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t0)
    return best


def test_heavy_leaves_native_tree_beats_padding(hodlr):
    """solver_irregular_part.cc with -heavy 1 of four shards: leaf 640 on the
    first subtree, 64 on the others, five levels each, rank 16 throughout."""
    m, L, r, k, heavy = 64, 5, 16, 8, 10
    shapes = [(m * heavy, L, r)] + [(m, L, r)] * 3
    tp = P.tree_problem(2, shapes, [r] * 6, nrhs=k, seed=5)
    t = make_tree(hodlr, tp, nrhs=k)
    u, sizes, n_pad = _padded_uniform(hodlr, tp, m * heavy, k)
    assert 3 * tp.n < n_pad                         # 26,624 rows against 81,920

    Bd = to_dev(tp.B)
    Bp = torch.empty((k, n_pad), dtype=torch.float64, device="cuda").t()

    def native():
        t.factor()
        Bd.copy_(to_dev(tp.B))
        t.solve(Bd)

    def padded():
        u.factor()
        hodlr.pad_rows(sizes, m * heavy, to_dev(tp.B), Bp)
        torch.cuda.synchronize()
        u.solve(Bp)

    native_s, padded_s = _best_seconds(native), _best_seconds(padded)
    X = to_host(Bd)
    Xp = torch.empty((k, tp.n), dtype=torch.float64, device="cuda").t()
    hodlr.unpad_rows(sizes, m * heavy, Bp, Xp)
    assert rel(X, to_host(Xp)) < 1e-11
    R = tp.B - tp.matvec(X)
    assert np.linalg.norm(R) / np.linalg.norm(tp.B) < 1e-12
    print("heavy leaves: native %d rows %.2f ms, padded %d rows %.2f ms"
          % (tp.n, native_s * 1e3, n_pad, padded_s * 1e3))
    assert native_s < padded_s
    t.close()
    u.close()
