"""Seeded HODLR test problems (TEST INFRASTRUCTURE ONLY).

Two families:

* :func:`reference_problem` -- fastSolver2's own inputs: uniform [0,1) drand48
  streams, one seed per leaf partition, D shifted by +1e3, one U and one V
  shared by every level (src/matrix.cc:250-297, src/tasks/dense_block.cc:63-75,
  spmd_driver/solver.cc:75-86, tests/test.cc:552-557).  The time(NULL) master
  seeds of the reference are replaced by fixed ones.
* :func:`gaussian_problem` -- the Gaussian workloads of the benchmark
  configurations: leaf blocks G/sqrt(m) + shift*I, off-diagonal factors
  N(0,1)/sqrt(n_block) drawn independently per level, optionally with
  orthonormalised factors and a singular-value profile s_i = 10^(-decay*i/r).

A problem's matrix is A = blockdiag(K_leaf) + sum over nodes p at depth l of
U^(l)_c0 diag(s^(l)) V^(l)_c1^T (block (c0,c1)) and U^(l)_c1 diag(s^(l))
V^(l)_c0^T (block (c1,c0)), c0/c1 the children of p.
"""
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import oracle


@dataclass
class Problem:
    leaf: int
    levels: int
    rank: int
    K: np.ndarray                 # N x m, leaf i at rows i*m (the KTree region)
    U: List[np.ndarray]           # per level, N x r
    V: List[np.ndarray]           # per level, N x r
    s: Optional[List[np.ndarray]]  # per level, r (None = all ones)
    B: np.ndarray                 # N x k

    @property
    def n(self):
        return self.leaf << self.levels

    @property
    def nrhs(self):
        return self.B.shape[1]

    def leaf_block(self, i):
        m = self.leaf
        return self.K[i * m:(i + 1) * m, :]

    def dense(self):
        """The full N x N matrix (small problems only)."""
        N, m, L = self.n, self.leaf, self.levels
        A = np.zeros((N, N))
        for i in range(1 << L):
            A[i * m:(i + 1) * m, i * m:(i + 1) * m] = self.leaf_block(i)
        for l in range(L):
            h = N >> (l + 1)
            s = self.s[l] if self.s is not None else np.ones(self.rank)
            for p in range(1 << l):
                c0 = slice(2 * p * h, (2 * p + 1) * h)
                c1 = slice((2 * p + 1) * h, (2 * p + 2) * h)
                A[c0, c1] = (self.U[l][c0] * s) @ self.V[l][c1].T
                A[c1, c0] = (self.U[l][c1] * s) @ self.V[l][c0].T
        return A


def reference_problem(leaf, levels, rank, nrhs=1, master=20240601, offset=1000):
    """The reference's uniform-drand48 problem with shared U and V."""
    nPart = 1 << levels
    vseeds = oracle.seeds(master + 0, nPart)
    useeds = oracle.seeds(master + 1, nPart)
    bseeds = oracle.seeds(master + 2, nPart)
    dseeds = oracle.seeds(master + 3, nPart)
    V = oracle.rand_matrix(vseeds, leaf, rank)
    U = oracle.rand_matrix(useeds, leaf, rank)
    B = oracle.rand_matrix(bseeds, leaf, nrhs)
    K = oracle.dense_blocks(useeds, vseeds, dseeds, leaf, rank, offset)
    return Problem(leaf, levels, rank, K, [U] * levels, [V] * levels, None, B)


def _orthonormal_blocks(X, nblocks):
    """QR-orthonormalise each of the nblocks row blocks of X."""
    out = np.empty_like(X)
    h = X.shape[0] // nblocks
    for b in range(nblocks):
        q, _ = np.linalg.qr(X[b * h:(b + 1) * h])
        out[b * h:(b + 1) * h] = q
    return out


def gaussian_problem(leaf, levels, rank, nrhs=1, seed=0, shift=4.0,
                     orthonormal=False, decay=None):
    """Gaussian HODLR problem (benchmark configurations' generators)."""
    rng = np.random.default_rng(seed)
    N = leaf << levels
    nleaf = 1 << levels
    G = rng.standard_normal((nleaf, leaf, leaf)) / np.sqrt(leaf)
    G += shift * np.eye(leaf)[None]
    K = np.asfortranarray(G.reshape(N, leaf))
    U, V = [], []
    for l in range(levels):
        nb = N >> (l + 1)
        u = rng.standard_normal((N, rank))
        v = rng.standard_normal((N, rank))
        if orthonormal:
            u = _orthonormal_blocks(u, 2 << l)
            v = _orthonormal_blocks(v, 2 << l)
        else:
            u /= np.sqrt(nb)
            v /= np.sqrt(nb)
        U.append(np.asfortranarray(u))
        V.append(np.asfortranarray(v))
    s = None
    if decay is not None:
        sv = 10.0 ** (-decay * np.arange(rank) / rank)
        s = [sv.copy() for _ in range(levels)]
    B = np.asfortranarray(rng.standard_normal((N, nrhs)))
    return Problem(leaf, levels, rank, K, U, V, s, B)


def rel_residual(prob, X, B=None):
    """||B - A X||_F / ||B||_F with A X from the FP64 HODLR matvec."""
    B = prob.B if B is None else B
    R = B - oracle.hodlr_matvec(prob, X)
    return np.linalg.norm(R) / np.linalg.norm(B)
