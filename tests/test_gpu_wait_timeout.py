"""A bounded device wait that runs out (no GPU fault, no hang).

The FP32 row-reduction kernels (on the tensor cores, and on the FMA pipe with
HODLR_NO_TCGEN05=1) wait on an mbarrier for each stage's TMA copies, with a
clock budget.  The test hook hodlr_debug_wait_fault makes one
CTA skip issuing one stage's copies, so nothing ever completes that wait: the
CTA's wait ends by its (short) budget, it records HODLR_ERR_TIMEOUT with its
index, waits for its own copies in flight and returns.  The factorisation
reports the error, and the same handle, with the hook off, then factors and
solves to the same bits as a fresh handle: the context stays usable.
"""
import pytest
import torch

pytestmark = pytest.mark.gpu

M, L, R, K = 128, 7, 32, 64
N = M << L


def colmajor(rows, cols):
    return torch.empty((cols, rows), dtype=torch.float64, device="cuda").t()


def mixed_solver(fs):
    s = fs.Solver(N, M, L, R, nrhs_max=K, precision=fs.PREC_MIXED, refine_tol=1e-12)
    B0 = colmajor(N, K)
    s.generate(31, shift=1.5, orthonormal=True, decay=6.0, B=B0)
    torch.cuda.synchronize()
    return s, B0


def solve(s, B0):
    X = colmajor(N, K)
    X.copy_(B0)
    info = s.solve(X)
    return X, info


@pytest.mark.parametrize("no_tc", ["0", "1"])
@pytest.mark.parametrize("cta,stage", [(1, 0), (0, 2)])
def test_reduce_wait_runs_out_and_reports_timeout(hodlr, cta, stage, no_tc, monkeypatch):
    monkeypatch.setenv("HODLR_NO_TCGEN05", no_tc)
    s, B0 = mixed_solver(hodlr)
    hodlr.debug_wait_fault(cta, stage, budget_cycles=200000)
    try:
        with pytest.raises(hodlr.HodlrError) as e:
            s.factor()
    finally:
        hodlr.debug_wait_fault(-1)
    assert e.value.code == hodlr.HODLR_ERR_TIMEOUT
    assert "(index %d)" % cta in str(e.value)
    s.factor()
    X, info = solve(s, B0)
    assert info.rel_residual <= 1e-12
    fresh, B1 = mixed_solver(hodlr)
    assert torch.equal(B0, B1)
    fresh.factor()
    Y, info2 = solve(fresh, B1)
    assert torch.equal(X, Y) and info.iterations == info2.iterations
    s.close()
    fresh.close()


def test_wait_fault_off_leaves_results_unchanged(hodlr):
    """With the hook pointed at a CTA index beyond every launch's grid, nothing changes."""
    s, B0 = mixed_solver(hodlr)
    s.factor()
    X, _ = solve(s, B0)
    hodlr.debug_wait_fault(1 << 30, 0, budget_cycles=200000)
    try:
        s.factor()
        Y, info = solve(s, B0)
    finally:
        hodlr.debug_wait_fault(-1)
    assert torch.equal(X, Y) and info.rel_residual <= 1e-12
    s.close()
