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


@dataclass
class TreeProblem:
    """An irregular tree: 2^T uniform subtrees (their own leaf, depth, rank)
    under T top levels; top node p = 2^l - 1 + q couples its children c0, c1
    by A[c0,c1] = U_c0 V_c1^T (rank ranks[2p]) and A[c1,c0] = U_c1 V_c0^T
    (rank ranks[2p+1]).  Uc[(l, q, h)] is U of child h (its rows x its own
    rank), Vc[(l, q, h)] its V (its rows x the sibling's rank)."""
    top_levels: int
    subs: List[Problem]
    ranks: List[int]
    Uc: dict
    Vc: dict
    B: np.ndarray

    @property
    def offsets(self):
        return np.concatenate([[0], np.cumsum([s.n for s in self.subs])]).astype(int).tolist()

    @property
    def n(self):
        return self.offsets[-1]

    def child_leaves(self, l, q, h):
        span = 1 << (self.top_levels - 1 - l)
        return (2 * q + h) * span, (2 * q + h + 1) * span

    def child_rows(self, l, q, h):
        j0, j1 = self.child_leaves(l, q, h)
        return slice(self.offsets[j0], self.offsets[j1])

    def u_rank(self, l, j):
        """Rank of the depth-l coupling U on the rows of subtree j."""
        T = self.top_levels
        p = (1 << l) - 1 + (j >> (T - l))
        return self.ranks[2 * p + ((j >> (T - 1 - l)) & 1)]

    def dense(self):
        A = np.zeros((self.n, self.n))
        off = self.offsets
        for j, s in enumerate(self.subs):
            A[off[j]:off[j + 1], off[j]:off[j + 1]] = s.dense()
        for l in range(self.top_levels):
            for q in range(1 << l):
                c0, c1 = self.child_rows(l, q, 0), self.child_rows(l, q, 1)
                A[c0, c1] = self.Uc[(l, q, 0)] @ self.Vc[(l, q, 1)].T
                A[c1, c0] = self.Uc[(l, q, 1)] @ self.Vc[(l, q, 0)].T
        return A

    def matvec(self, X):
        """A X from the representation (subtree products by the oracle)."""
        X = np.asarray(X, dtype=np.float64).reshape(self.n, -1)
        Y = np.zeros_like(X)
        off = self.offsets
        for j, s in enumerate(self.subs):
            Y[off[j]:off[j + 1]] = oracle.hodlr_matvec(s, X[off[j]:off[j + 1]])
        for l in range(self.top_levels):
            for q in range(1 << l):
                c0, c1 = self.child_rows(l, q, 0), self.child_rows(l, q, 1)
                Y[c0] += self.Uc[(l, q, 0)] @ (self.Vc[(l, q, 1)].T @ X[c1])
                Y[c1] += self.Uc[(l, q, 1)] @ (self.Vc[(l, q, 0)].T @ X[c0])
        return Y


def tree_problem(top_levels, shapes, coupling_ranks, nrhs=1, seed=0, shift=4.0, orthonormal=False, decay=None):
    """Gaussian irregular tree: subtree j is gaussian_problem(*shapes[j])
    (leaf, levels, rank), the coupling bases N(0,1)/sqrt(child rows)."""
    rng = np.random.default_rng(seed)
    subs = [gaussian_problem(m, L, r, nrhs=1, seed=seed * 1000 + 1 + j, shift=shift, orthonormal=orthonormal,
                             decay=decay) for j, (m, L, r) in enumerate(shapes)]
    tp = TreeProblem(top_levels, subs, list(coupling_ranks), {}, {}, None)
    for l in range(top_levels):
        for q in range(1 << l):
            p = (1 << l) - 1 + q
            for h in (0, 1):
                rows = tp.child_rows(l, q, h)
                nr = rows.stop - rows.start
                ru, rv = coupling_ranks[2 * p + h], coupling_ranks[2 * p + 1 - h]
                tp.Uc[(l, q, h)] = np.asfortranarray(rng.standard_normal((nr, ru)) / np.sqrt(nr))
                tp.Vc[(l, q, h)] = np.asfortranarray(rng.standard_normal((nr, rv)) / np.sqrt(nr))
    tp.B = np.asfortranarray(rng.standard_normal((tp.n, nrhs)))
    return tp


def rel_residual(prob, X, B=None):
    """||B - A X||_F / ||B||_F with A X from the FP64 HODLR matvec."""
    B = prob.B if B is None else B
    R = B - oracle.hodlr_matvec(prob, X)
    return np.linalg.norm(R) / np.linalg.norm(B)
