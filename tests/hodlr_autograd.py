"""torch.autograd.Function over the C ABI -- a TEST HARNESS ONLY.

x = A^{-1} b for the HODLR matrix A(D, U, V, s); backward calls the
library's hand-written adjoint sweep (hodlr_adjoint: lambda = A^{-T} g, then
the rank-k outer-product gradients), so torch's autograd checks (gradcheck,
finite differences) exercise the CUDA adjoint end to end.

Tensor layouts (CUDA, float64): b (N, k); D (nleaf, m, m) with D[i] the leaf
block (row-major torch view of the column-major [leaf][m][m] buffer is
transposed: D[i].T is what the library reads); U, V (L, N, r); s (L, r).
"""
import torch

import fastsolver2_gb300 as fs


def _colmajor_2d(t):
    return t.t().contiguous().t()


class HodlrSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, b, D, U, V, s, leaf, precision=fs.PREC_FP64):
        L, N, r = U.shape
        k = b.shape[1]
        solver = fs.Solver(N, leaf, L, r, nrhs_max=k, precision=precision)
        # leaf blocks: the library wants column-major m x m per leaf
        Dcm = D.transpose(1, 2).contiguous()          # memory = column-major blocks
        Ucm = [U[l].t().contiguous() for l in range(L)]   # (r, N) row-major = (N, r) column-major
        Vcm = [V[l].t().contiguous() for l in range(L)]
        X = _colmajor_2d(b.detach().clone())
        s = s.contiguous()
        # the library works on its own non-blocking stream: the torch kernels
        # that made its inputs must have finished before it reads them
        torch.cuda.synchronize()
        solver.set_leaf_blocks(Dcm.reshape(-1), ld=leaf, leaf_stride=leaf * leaf)
        for l in range(L):
            solver.set_lowrank(l, Ucm[l].t(), Vcm[l].t(), s[l])
        solver.factor()
        solver.solve(X)
        ctx.solver = solver
        ctx.save_for_backward(X)
        ctx.shape = (L, N, r, leaf, k)
        return X.clone()

    @staticmethod
    def backward(ctx, gx):
        (X,) = ctx.saved_tensors
        L, N, r, leaf, k = ctx.shape
        dev = X.device
        g = _colmajor_2d(gx.contiguous())
        db = torch.empty((k, N), dtype=torch.float64, device=dev).t()
        dD = torch.empty((N // leaf) * leaf * leaf, dtype=torch.float64, device=dev)
        dU = torch.empty(L * N * r, dtype=torch.float64, device=dev)
        dV = torch.empty(L * N * r, dtype=torch.float64, device=dev)
        ds = torch.empty(L * r, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()   # g is made by torch kernels; the library reads it on its own stream
        ctx.solver.adjoint(X, g, db=db, dD=dD, dU=dU, dV=dV, ds=ds)
        nleaf = N // leaf
        dD = dD.reshape(nleaf, leaf, leaf).transpose(1, 2)   # back to D[i] row-major indexing
        dU = dU.reshape(L, r, N).transpose(1, 2)
        dV = dV.reshape(L, r, N).transpose(1, 2)
        return db, dD, dU, dV, ds.reshape(L, r), None, None


def hodlr_solve(b, D, U, V, s, leaf):
    return HodlrSolve.apply(b, D, U, V, s, leaf)
