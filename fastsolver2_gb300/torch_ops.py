"""torch operators over the HODLR library: ``fastsolver2::hodlr_solve`` and
its adjoint ``fastsolver2::hodlr_solve_backward``, registered with
torch.library so they work with autograd, the fake-tensor shape machinery
(torch.compile traces them as opaque calls) and ``torch.ops``.

    x = hodlr_solve(b, D, U, V, s, leaf, precision=PREC_FP64)

solves A x = b for the HODLR matrix A = blockdiag(D) + sum over the nodes
of the off-diagonal couplings U diag(s) V^T, one (leaf, levels, rank)
geometry per call (fastSolver2's HMatrix::init + HMatrix::solve,
src/hmatrix.cc:22-96, as one functional op).  Layouts (CUDA, float64):

* b: (N, k) right-hand sides;
* D: (nleaf, m, m), D[i] the i-th leaf block (row-major torch indexing);
* U, V: (L, N, r), level l's bases (U[l] rows c*N/2^(l+1).. couple child c);
* s: (L, r) the singular-value profile of each level.

The backward (the gradients of a loss with respect to b, D, U, V and s) is
the library's adjoint sweep (hodlr_adjoint: lambda = A^{-T} g on the FP64
factorisation, then the rank-k outer-product gradients).  Both ops factor
the matrix from their inputs; the forward's factorisation is not kept
between the two, so a backward costs one FP64 factorisation plus a
transposed solve.  Inputs must be CUDA float64 tensors; there is no CPU
implementation.
"""
from typing import Tuple

import torch

from . import PREC_FP64, Solver

_NS = "fastsolver2"


def _factored(D, U, V, s, leaf, k, precision):
    """A factored Solver for the HODLR matrix given in op layout."""
    L, N, r = U.shape
    # the library works on torch's current stream, ordered with the torch
    # kernels that made its inputs; the copies stay alive until factor()
    # (which synchronises) has run
    solver = Solver(N, leaf, L, r, nrhs_max=k, precision=precision, stream=torch.cuda.current_stream().cuda_stream)
    keep = [D.transpose(1, 2).contiguous()]          # column-major leaf blocks
    solver.set_leaf_blocks(keep[0].reshape(-1), ld=leaf, leaf_stride=leaf * leaf)
    for l in range(L):
        Ul, Vl, sl = U[l].t().contiguous().t(), V[l].t().contiguous().t(), s[l].contiguous()
        keep += [Ul, Vl, sl]
        solver.set_lowrank(l, Ul, Vl, sl)
    solver.factor()
    return solver


def _colmajor_copy(t):
    """A new column-major copy of the 2-D tensor t (never a view of t: the
    library solves in place)."""
    out = torch.empty((t.shape[1], t.shape[0]), dtype=t.dtype, device=t.device).t()
    out.copy_(t)
    return out


def _check(b, D, U, V, s):
    for t in (b, D, U, V, s):
        if not (t.is_cuda and t.dtype == torch.float64):
            raise TypeError("fastsolver2 ops take CUDA float64 tensors")


@torch.library.custom_op(_NS + "::hodlr_solve", mutates_args=())
def hodlr_solve(b: torch.Tensor, D: torch.Tensor, U: torch.Tensor, V: torch.Tensor, s: torch.Tensor, leaf: int,
                precision: int = PREC_FP64) -> torch.Tensor:
    _check(b, D, U, V, s)
    solver = _factored(D, U, V, s, leaf, b.shape[1], precision)
    X = _colmajor_copy(b.detach())                     # solved in place
    solver.solve(X)
    solver.close()
    return torch.empty_like(b).copy_(X)                # b's layout (as the fake implementation gives)


@hodlr_solve.register_fake
def _(b, D, U, V, s, leaf, precision=PREC_FP64):
    return torch.empty_like(b)


@torch.library.custom_op(_NS + "::hodlr_solve_backward", mutates_args=())
def hodlr_solve_backward(x: torch.Tensor, g: torch.Tensor, D: torch.Tensor, U: torch.Tensor, V: torch.Tensor,
                         s: torch.Tensor, leaf: int) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor,
                                                              torch.Tensor, torch.Tensor]:
    _check(g, D, U, V, s)
    L, N, r = U.shape
    k, nleaf, dev = x.shape[1], N // leaf, x.device
    solver = _factored(D, U, V, s, leaf, k, PREC_FP64)
    X = _colmajor_copy(x.detach())
    G = _colmajor_copy(g.detach())
    db = torch.empty((k, N), dtype=torch.float64, device=dev).t()
    dD = torch.empty(nleaf * leaf * leaf, dtype=torch.float64, device=dev)
    dU = torch.empty(L * N * r, dtype=torch.float64, device=dev)
    dV = torch.empty(L * N * r, dtype=torch.float64, device=dev)
    ds = torch.empty(L * r, dtype=torch.float64, device=dev)
    solver.adjoint(X, G, db=db, dD=dD, dU=dU, dV=dV, ds=ds)
    solver.close()
    return (db.contiguous(), dD.reshape(nleaf, leaf, leaf).transpose(1, 2).contiguous(),
            dU.reshape(L, r, N).transpose(1, 2).contiguous(), dV.reshape(L, r, N).transpose(1, 2).contiguous(),
            ds.reshape(L, r))


@hodlr_solve_backward.register_fake
def _(x, g, D, U, V, s, leaf):
    return (torch.empty_like(x), torch.empty_like(D), torch.empty_like(U), torch.empty_like(V), torch.empty_like(s))


def _setup_context(ctx, inputs, output):
    b, D, U, V, s, leaf, precision = inputs
    ctx.save_for_backward(D, U, V, s, output)
    ctx.leaf = leaf


def _backward(ctx, gx):
    D, U, V, s, x = ctx.saved_tensors
    db, dD, dU, dV, ds = hodlr_solve_backward(x, gx, D, U, V, s, ctx.leaf)
    return db, dD, dU, dV, ds, None, None


hodlr_solve.register_autograd(_backward, setup_context=_setup_context)
