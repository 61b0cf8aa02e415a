"""Ragged batches (hodlr_batch_*) through the C ABI.

Every system of a batch is checked on its own: against the oracle's solve of
the same problem (FP64: 1e-12 relative), against its own relative residual
(mixed: the refinement target 1e-12), and against a standalone handle built
from the same seeded generator (the batch stacks systems that share leaf size
and rank into one forest; a system's solution must not depend on its
neighbours).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle import problems as P

pytestmark = pytest.mark.gpu

DD = dict(dtype=torch.float64, device="cuda")


def to_dev(a):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        return torch.from_numpy(a.copy()).cuda()
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()


def to_host(t):
    return np.asfortranarray(t.t().cpu().numpy().T)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


# (leaf, levels, rank, nrhs): three forests of unequal depths, a one-leaf
# system, repeated shapes, and rank > leaf / 2 in a shallow tree
RAGGED = [(32, 3, 4, 2), (16, 4, 4, 1), (32, 1, 4, 3), (64, 2, 8, 1), (32, 3, 4, 1), (16, 0, 4, 2),
          (64, 4, 8, 2), (16, 2, 4, 1), (32, 0, 4, 1), (64, 1, 8, 3)]


def _problems(shapes, seed0=100, **kw):
    return [P.gaussian_problem(m, L, r, nrhs=k, seed=seed0 + i, **kw) for i, (m, L, r, k) in enumerate(shapes)]


def _load(fs, probs, precision, **kw):
    b = fs.Batch([(p.n, p.leaf, p.levels, p.rank, p.nrhs) for p in probs], precision=precision, **kw)
    keep = []
    for i, p in enumerate(probs):
        K = to_dev(p.K)
        b.set_leaf_blocks(i, K)
        keep.append(K)
        for l in range(p.levels):
            U, V = to_dev(p.U[l]), to_dev(p.V[l])
            sv = to_dev(p.s[l]) if p.s is not None else None
            b.set_lowrank(i, l, U, V, sv)
            keep += [U, V, sv]
    torch.cuda.synchronize()
    return b


def test_fp64_ragged_batch_matches_oracle(hodlr):
    probs = _problems(RAGGED)
    b = _load(hodlr, probs, hodlr.PREC_FP64)
    nforests, _, _ = b.stats()
    assert nforests == 3
    b.factor()
    for rep in range(2):  # the second solve replays the captured graph
        Bs = [to_dev(p.B) for p in probs]
        torch.cuda.synchronize()
        info = b.solve(Bs)
        for i, p in enumerate(probs):
            Xo, _, _ = O.hsolve_general(p, p.B)
            X = to_host(Bs[i])
            assert info[i].status == hodlr.HODLR_OK
            assert rel(X, Xo) < 1e-12, (rep, i, rel(X, Xo))
            assert P.rel_residual(p, X) < 1e-10


def test_mixed_ragged_batch_reaches_tolerance(hodlr):
    probs = _problems(RAGGED, seed0=300, decay=2.0)
    b = _load(hodlr, probs, hodlr.PREC_MIXED, refine_tol=1e-12)
    b.factor()
    for rep in range(2):
        Bs = [to_dev(p.B) for p in probs]
        torch.cuda.synchronize()
        info = b.solve(Bs)
        for i, p in enumerate(probs):
            X = to_host(Bs[i])
            res = P.rel_residual(p, X)
            # the per-column refinement test bounds the Frobenius residual too
            assert res <= 1.5e-12, (rep, i, res)
            assert 0.0 <= info[i].rel_residual <= 1e-12
            assert info[i].status == hodlr.HODLR_OK


@pytest.mark.parametrize("precision", [0, 1])
def test_generated_batch_matches_standalone_handles(hodlr, precision):
    shapes = [(128, 4, 16, 3), (64, 5, 8, 1), (128, 2, 16, 2), (256, 2, 32, 4), (64, 3, 8, 8), (128, 5, 16, 1)]
    systems = [(m << L, m, L, r, k) for m, L, r, k in shapes]
    b = hodlr.Batch(systems, precision=precision)
    Bs = [torch.empty((k, n), **DD).t() for n, m, L, r, k in systems]
    b.generate(77, shift=4.0, Bs=Bs)
    B0 = [x.clone() for x in Bs]
    b.factor()
    torch.cuda.synchronize()
    info = b.solve(Bs)
    for i, (n, m, L, r, k) in enumerate(systems):
        s = hodlr.Solver(n, m, L, r, nrhs_max=k, precision=precision)
        Bi = torch.empty((k, n), **DD).t()
        s.generate(77 + i, shift=4.0, orthonormal=False, decay=0.0, B=Bi)
        assert torch.equal(Bi, B0[i])   # same seeded generator, same inputs
        s.factor()
        s.solve(Bi)
        d = (Bs[i] - Bi).norm() / Bi.norm()
        assert d < (1e-13 if precision == 0 else 1e-11), (i, float(d))
        if precision == 1:
            assert info[i].rel_residual <= 1e-12


def test_batch_reports_the_failing_system(hodlr):
    probs = _problems(RAGGED[:4], seed0=500)
    b = _load(hodlr, probs, hodlr.PREC_FP64)
    b.factor()
    Bs = [to_dev(p.B) for p in probs]
    Bs[2][1, 0] = float("nan")
    torch.cuda.synchronize()
    with pytest.raises(hodlr.HodlrError) as e:
        b.solve(Bs)
    assert e.value.code == hodlr.HODLR_ERR_NONFINITE_INPUT
    assert "system 2" in str(e.value)


def test_batch_rejects_bad_systems(hodlr):
    with pytest.raises(hodlr.HodlrError):
        hodlr.Batch([(100, 16, 2, 4, 1)])          # n != leaf * 2^levels
    with pytest.raises(hodlr.HodlrError):
        hodlr.Batch([(64, 16, 2, 0, 1)])           # rank 0
    b = hodlr.Batch([(64, 16, 2, 4, 1)])
    with pytest.raises(hodlr.HodlrError):
        b.factor()                                 # inputs not set


def test_batch_autotune_then_solve(hodlr):
    probs = _problems(RAGGED[:6], seed0=700)
    b = _load(hodlr, probs, hodlr.PREC_MIXED)
    tunes = b.autotune()
    assert len(tunes) == b.stats()[0]
    for t in tunes:
        assert t["red_ctas_per_sm"] in (2, 4, 8) and t["update_tile_rows"] in (0, 64) and t["ms"] > 0
        assert t["cap_warps"] in (0, 8, 16) and t["update_tc_shape"] in (0, 1, 2) and t["leaf_apply"] in (0, 1)
    b.factor()
    Bs = [to_dev(p.B) for p in probs]
    torch.cuda.synchronize()
    b.solve(Bs)
    for i, p in enumerate(probs):
        assert P.rel_residual(p, to_host(Bs[i])) <= 1.5e-12
