"""The package's torch operators (fastsolver2::hodlr_solve and its adjoint):
registration and shapes on the CPU; on the GPU, the solution against a dense
FP64 solve, the gradients against central differences and against the
adjoint test harness."""
import numpy as np
import pytest
import torch

from oracle import problems as P


def test_ops_are_registered_and_trace_shapes():
    import fastsolver2_gb300.torch_ops  # noqa: F401  (registers the ops)
    assert hasattr(torch.ops.fastsolver2, "hodlr_solve")
    assert hasattr(torch.ops.fastsolver2, "hodlr_solve_backward")
    from torch._subclasses.fake_tensor import FakeTensorMode
    with FakeTensorMode():
        b = torch.empty(256, 3, dtype=torch.float64)
        D = torch.empty(8, 32, 32, dtype=torch.float64)
        U = torch.empty(3, 256, 4, dtype=torch.float64)
        s = torch.empty(3, 4, dtype=torch.float64)
        x = torch.ops.fastsolver2.hodlr_solve(b, D, U, U, s, 32)
        assert x.shape == (256, 3)
        g = torch.ops.fastsolver2.hodlr_solve_backward(x, x, D, U, U, s, 32)
        assert [t.shape for t in g] == [b.shape, D.shape, U.shape, U.shape, s.shape]


def _op_inputs(pr):
    dev = dict(dtype=torch.float64, device="cuda")
    nleaf, m = 1 << pr.levels, pr.leaf
    D = torch.tensor(np.stack([pr.leaf_block(i) for i in range(nleaf)]), **dev)
    U = torch.tensor(np.stack(pr.U), **dev)
    V = torch.tensor(np.stack(pr.V), **dev)
    s = torch.tensor(np.stack(pr.s), **dev)
    b = torch.tensor(pr.B, **dev)
    return b, D, U, V, s


@pytest.mark.gpu
def test_hodlr_solve_op_forward_and_gradients(hodlr):
    from fastsolver2_gb300.torch_ops import hodlr_solve
    from tests.hodlr_autograd import HodlrSolve
    pr = P.gaussian_problem(32, 3, 4, nrhs=2, seed=12, orthonormal=True, decay=2.0, shift=3.0)
    b, D, U, V, s = _op_inputs(pr)
    x = hodlr_solve(b, D, U, V, s, pr.leaf)
    xd = np.linalg.solve(pr.dense(), pr.B)
    assert np.linalg.norm(x.cpu().numpy() - xd) / np.linalg.norm(xd) < 1e-12
    # gradients of 0.5 ||x||^2: the op's against the harness Function's
    ins = [t.clone().requires_grad_(True) for t in (b, D, U, V, s)]
    (0.5 * hodlr_solve(*ins, pr.leaf).pow(2).sum()).backward()
    ref = [t.clone().requires_grad_(True) for t in (b, D, U, V, s)]
    (0.5 * HodlrSolve.apply(*ref, pr.leaf).pow(2).sum()).backward()
    for a, c in zip(ins, ref):
        assert torch.allclose(a.grad, c.grad, rtol=1e-10, atol=1e-12)
    # and against central differences for b and s (few entries: gradcheck)
    f = lambda bb, ss: hodlr_solve(bb, D, U, V, ss, pr.leaf)
    assert torch.autograd.gradcheck(f, (b.clone().requires_grad_(True), s.clone().requires_grad_(True)),
                                    eps=1e-6, atol=1e-7, rtol=1e-6)


@pytest.mark.gpu
def test_hodlr_solve_op_mixed_precision(hodlr):
    from fastsolver2_gb300.torch_ops import hodlr_solve
    pr = P.gaussian_problem(64, 3, 8, nrhs=3, seed=5, orthonormal=True, decay=6.0, shift=1.5)
    b, D, U, V, s = _op_inputs(pr)
    x = hodlr_solve(b, D, U, V, s, pr.leaf, hodlr.PREC_MIXED)
    assert P.rel_residual(pr, x.cpu().numpy()) < 2e-12
