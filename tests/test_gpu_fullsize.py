"""The benchmark configurations at full size (N = 2^20, leaf 128, 13 levels,
rank 32, 64 right-hand sides) against the reference's arithmetic on the host.

* FP64, reference-structured inputs (the reference's drand48 streams, leaf
  blocks U V^T + diag(D + 1e3), one U and one V for every level): the drop-in
  entry point hodlr_hsolve against fastSolver2's hsolve restated with its
  dgemm_/dgesv_ calls on OpenBLAS (bitwise the reference's own build on that
  BLAS, tests/test_oracle.py), threaded the way the reference's index launch
  splits the tree.  Solution, transformed bases and leaf LU within 1e-12
  relative; relative residual <= 1e-10 (the FP64 parity bar).
* Mixed precision with FP64 refinement on the ill-conditioned configuration
  (orthonormal factors, s_i = 10^(-6 i/32), leaf shift 1.5): the refinement
  target 1e-12 checked by an FP64 residual computed on the host from the
  handle's exact inputs (the oracle's HODLR product on OpenBLAS), not by the
  library's own residual.

Each test holds ~6 GB on the device and ~12 GB on the host and takes tens of
seconds, most of it host BLAS.
"""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

M, L, R, K = 128, 13, 32, 64
NP = 1 << L
N = M * NP


def colmajor(rows, cols):
    return torch.empty((cols, rows), dtype=torch.float64, device="cuda").t()


def host(t):
    """Column-major device tensor -> Fortran-ordered numpy array."""
    return np.asfortranarray(t.t().cpu().numpy().T)


def threads():
    return os.cpu_count() or 1


@pytest.fixture(scope="module")
def blas():
    if O.blas_lib() is None:
        pytest.skip("scipy's OpenBLAS is not available on this host")
    return O


def test_fp64_hsolve_full_size_matches_reference_hsolve(hodlr, blas):
    master = 4242
    vs, us, bs, ds = (hodlr.draw_seeds(master + i, NP) for i in range(4))
    gen = hodlr.Solver(N, M, L, R)
    gen.set_seeded(us, vs, ds, offset=1000.0)
    Kd = colmajor(N, M)                       # KTree region: leaf i at rows i*m, LD = N
    gen.get_inputs(D=Kd, ld=N, leaf_stride=M)
    gen.close()
    Ud, Vd = colmajor(N, R), colmajor(N, R)
    hodlr.rand_matrix(us, M, Ud)
    hodlr.rand_matrix(vs, M, Vd)
    Wd = colmajor(N, K + L * R)               # UTree region [b | U | ... | U]
    hodlr.rand_matrix(bs, M, Wd[:, :K])
    for l in range(L):
        Wd[:, K + l * R:K + (l + 1) * R].copy_(Ud)
    torch.cuda.synchronize()
    Kh, Wh, Vh = host(Kd), host(Wd), host(Vd)
    K0, B = Kh.copy(order="F"), Wh[:, :K].copy(order="F")
    U0 = Wh[:, K:K + R].copy(order="F")

    hodlr.hsolve(N, K, R, NP, N, Kd, Wd, Vd)            # the drop-in entry point, FP64, in place
    assert blas.blas_hsolve_mt(M, L, R, Kh, [Vh] * L, Wh, K, threads()) == 0

    Wg, Kg = host(Wd), host(Kd)
    X, Xr = Wg[:, :K], Wh[:, :K]
    assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) < 1e-12
    assert np.linalg.norm(Wg - Wh) / np.linalg.norm(Wh) < 1e-12      # x and every transformed basis
    assert np.linalg.norm(Kg - Kh) / np.linalg.norm(Kh) < 1e-12      # leaf LU factors
    Y = blas.blas_matvec(M, L, R, K0, [U0] * L, [Vh] * L, None, np.asfortranarray(X), threads())
    resid = (np.linalg.norm(B - Y, axis=0) / np.linalg.norm(B, axis=0)).max()
    assert resid <= 1e-10, resid


def test_mixed_full_size_refines_to_1e12_by_host_fp64_residual(hodlr, blas):
    s = hodlr.Solver(N, M, L, R, nrhs_max=K, precision=hodlr.PREC_MIXED, refine_tol=1e-12, refine_max_iter=10)
    B0 = colmajor(N, K)
    s.generate(20261204, shift=1.5, orthonormal=True, decay=6.0, B=B0)
    X = colmajor(N, K)
    X.copy_(B0)
    s.factor()
    info = s.solve(X)
    assert info.rel_residual <= 1e-12 and info.iterations >= 1
    Dh = colmajor(N, M)
    Uh, Vh = colmajor(N, L * R), colmajor(N, L * R)
    sh = torch.empty(L * R, dtype=torch.float64, device="cuda")
    s.get_inputs(D=Dh, ld=N, leaf_stride=M, U=Uh, V=Vh, s=sh)
    torch.cuda.synchronize()
    Kh, Uh, Vh, sh = host(Dh), host(Uh), host(Vh), sh.cpu().numpy()
    Xh, Bh = host(X), host(B0)
    s.close()
    Us = [Uh[:, l * R:(l + 1) * R] for l in range(L)]
    Vs = [Vh[:, l * R:(l + 1) * R] for l in range(L)]
    ss = [np.ascontiguousarray(sh[l * R:(l + 1) * R]) for l in range(L)]
    Y = blas.blas_matvec(M, L, R, Kh, Us, Vs, ss, Xh, threads())
    resid = (np.linalg.norm(Bh - Y, axis=0) / np.linalg.norm(Bh, axis=0)).max()
    assert resid <= 1e-12, (resid, info.rel_residual)
    # the library's own FP64-accurate residual estimate agrees with the host's
    assert abs(resid - info.rel_residual) <= 0.1 * resid, (resid, info.rel_residual)
