"""Adjoint sweep checks: torch.autograd.gradcheck through the C ABI at a small
size, and central finite differences (h = 1e-6, FP64) of L = 0.5 ||x||^2 with
respect to b, D_leaf, U, V and s at N = 2^18 (leaf 128, 11 levels, rank 24,
1 right-hand side).  The dense FP64 reference gradient at N = 2048 is in
test_gpu_solver.py::test_adjoint_matches_dense_gradient."""
import time

import pytest
import torch

import fastsolver2_gb300 as fs
from tests.hodlr_autograd import HodlrSolve

pytestmark = pytest.mark.gpu


def test_gradcheck_small(hodlr):
    torch.manual_seed(0)
    m, L, r, k = 8, 2, 2, 2
    N = m << L
    dd = dict(dtype=torch.float64, device="cuda")
    b = torch.randn(N, k, **dd, requires_grad=True)
    D = (torch.randn(1 << L, m, m, **dd) / m ** 0.5 + 3 * torch.eye(m, **dd)).requires_grad_()
    U = (torch.randn(L, N, r, **dd) * 0.3).requires_grad_()
    V = (torch.randn(L, N, r, **dd) * 0.3).requires_grad_()
    s = (torch.rand(L, r, **dd) + 0.5).requires_grad_()
    f = lambda b, D, U, V, s: HodlrSolve.apply(b, D, U, V, s, m)
    assert torch.autograd.gradcheck(f, (b, D, U, V, s), eps=1e-6, atol=1e-6, rtol=1e-5)


def _problem_tensors(N, m, L, r, k, seed):
    s = fs.Solver(N, m, L, r, nrhs_max=k)
    dd = dict(dtype=torch.float64, device="cuda")
    B = torch.empty((k, N), **dd).t()
    s.generate(seed, shift=4.0, orthonormal=False, decay=2.0, B=B)
    nleaf = N // m
    Dlib = torch.empty(nleaf * m * m, **dd)
    Ulib = torch.empty(L * N * r, **dd)
    Vlib = torch.empty(L * N * r, **dd)
    slib = torch.empty(L * r, **dd)
    s.get_inputs(D=Dlib, U=Ulib, V=Vlib, s=slib)
    torch.cuda.synchronize()
    D = Dlib.reshape(nleaf, m, m).transpose(1, 2).contiguous()
    U = Ulib.reshape(L, r, N).transpose(1, 2).contiguous()
    V = Vlib.reshape(L, r, N).transpose(1, 2).contiguous()
    return B.contiguous(), D, U, V, slib.reshape(L, r).contiguous()


def test_fd_and_cost_at_2_18(hodlr):
    m, L, r, k = 128, 11, 24, 1
    N = m << L
    b, D, U, V, s = _problem_tensors(N, m, L, r, k, seed=4)
    for _ in range(2):  # the second pass is timed (the first loads the kernels)
        params = [t.clone().requires_grad_() for t in (b, D, U, V, s)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x = HodlrSolve.apply(*params, m)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        loss = 0.5 * (x * x).sum()
        loss.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
    fwd, adj = t1 - t0, t2 - t1
    print("forward (factor+solve) %.1f ms, adjoint %.1f ms" % (1e3 * fwd, 1e3 * adj))
    assert adj <= 1.5 * fwd
    gen = torch.Generator(device="cuda").manual_seed(1)
    h = 1e-6
    with torch.no_grad():
        for idx, name in enumerate(["b", "D", "U", "V", "s"]):
            base = [t.detach() for t in (b, D, U, V, s)]
            d = torch.randn(base[idx].shape, dtype=torch.float64, device="cuda", generator=gen)
            if name == "D":  # perturb leaf blocks only on their entries (all are free parameters)
                d = d / m
            vals = []
            for sign in (1.0, -1.0):
                p = list(base)
                p[idx] = base[idx] + sign * h * d
                xp = HodlrSolve.apply(*p, m)
                vals.append(0.5 * float((xp * xp).sum()))
            fd = (vals[0] - vals[1]) / (2 * h)
            an = float((params[idx].grad * d).sum())
            assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-8), (name, fd, an)
