"""The working precision of the mixed path, justified numerically (CPU).

The mixed configuration's generator (orthonormalised per-block factors,
s_i = 10^(-6i/r), leaf shift 1.5) at N = 4096: a dense LU in FP32 refines to
a relative residual of 1e-12 in one correction, while factors whose inputs
are rounded to TF32 (11-bit significand, what a TF32 tensor-core GEMM sees)
or BF16 (8 bits) need three or more -- and on GB300 every extra correction
costs a full solve sweep plus an FP64-accurate residual, more than the FP32
low-rank GEMMs that tensor cores could shorten.  This is why the mixed path
computes in FP32 on the CUDA cores.
"""
import numpy as np
import scipy.linalg as sl

from oracle import problems as P


def _round_significand(X, bits):
    m, e = np.frexp(X)
    return np.ldexp(np.round(m * 2.0 ** bits) / 2.0 ** bits, e)


def _corrections(A, B, bits, tol=1e-12, cap=12):
    lu = sl.lu_factor(_round_significand(A, bits).astype(np.float32))
    x = sl.lu_solve(lu, B.astype(np.float32)).astype(np.float64)
    for it in range(cap + 1):
        r = B - A @ x
        if (np.linalg.norm(r, axis=0) / np.linalg.norm(B, axis=0)).max() <= tol:
            return it
        x = x + sl.lu_solve(lu, r.astype(np.float32)).astype(np.float64)
    return cap + 1


def test_fp32_factors_need_fewer_corrections_than_tf32_or_bf16():
    pr = P.gaussian_problem(128, 5, 32, nrhs=4, seed=3, shift=1.5, orthonormal=True, decay=6.0)
    A = pr.dense()
    fp32, tf32, bf16 = (_corrections(A, pr.B, bits) for bits in (24, 11, 8))
    assert fp32 <= 1
    assert tf32 >= 3 and bf16 >= tf32
