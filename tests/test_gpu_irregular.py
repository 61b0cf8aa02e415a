"""Trees with unequal leaf sizes (spmd_driver/solver_irregular_part.cc) and
unequal sibling ranks, solved by their exact embedding in the uniform tree:
leaves padded to the largest size with identity blocks, padded rows of U, V
and B zero (hodlr_pad_rows / hodlr_pad_leaf_blocks / hodlr_unpad_rows).
Checked against a dense FP64 solve of the unequal-leaf matrix."""
import numpy as np
import pytest
import torch

from tests.test_gpu_solver import to_dev, to_host

pytestmark = pytest.mark.gpu


def irregular_problem(sizes, levels, rank, nrhs, seed):
    rng = np.random.default_rng(seed)
    sizes = np.asarray(sizes)
    off = np.concatenate([[0], np.cumsum(sizes)])
    n = int(off[-1])
    A = np.zeros((n, n))
    blocks = []
    for i, m in enumerate(sizes):
        D = rng.standard_normal((m, m)) / np.sqrt(m) + 2.0 * np.eye(m)
        blocks.append(D)
        A[off[i]:off[i + 1], off[i]:off[i + 1]] = D
    U, V = [], []
    for l in range(levels):
        u = rng.standard_normal((n, rank)) / np.sqrt(n >> l)
        v = rng.standard_normal((n, rank)) / np.sqrt(n >> l)
        U.append(u)
        V.append(v)
        per = 1 << (levels - l - 1)  # leaves per child at depth l
        for p in range(1 << l):
            c0 = slice(off[2 * p * per], off[(2 * p + 1) * per])
            c1 = slice(off[(2 * p + 1) * per], off[(2 * p + 2) * per])
            A[c0, c1] += u[c0] @ v[c1].T
            A[c1, c0] += u[c1] @ v[c0].T
    B = rng.standard_normal((n, nrhs))
    return sizes, blocks, U, V, B, A


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("levels,m_max,rank,nrhs", [(3, 64, 8, 2), (4, 128, 16, 3)])
def test_unequal_leaf_sizes_by_padding(hodlr, precision, levels, m_max, rank, nrhs):
    rng = np.random.default_rng(levels)
    sizes = rng.integers(m_max // 2, m_max + 1, size=1 << levels)
    sizes[3] = m_max  # at least one full leaf; the others ragged
    sizes, blocks, U, V, B, A = irregular_problem(sizes, levels, rank, nrhs, seed=7 + levels)
    nleaf, n_pad = len(sizes), len(sizes) * m_max
    packed = torch.from_numpy(np.concatenate([b.ravel(order="F") for b in blocks])).cuda()
    Dp = torch.empty(nleaf * m_max * m_max, dtype=torch.float64, device="cuda")
    hodlr.pad_leaf_blocks(sizes, m_max, packed, Dp)
    s = hodlr.Solver(n_pad, m_max, levels, rank, nrhs_max=nrhs, precision=precision, refine_tol=1e-12)
    s.set_leaf_blocks(Dp, ld=m_max, leaf_stride=m_max * m_max)
    keep = []
    for l in range(levels):
        Up = torch.empty((rank, n_pad), dtype=torch.float64, device="cuda").t()
        Vp = torch.empty((rank, n_pad), dtype=torch.float64, device="cuda").t()
        hodlr.pad_rows(sizes, m_max, to_dev(U[l]), Up)
        hodlr.pad_rows(sizes, m_max, to_dev(V[l]), Vp)
        keep += [Up, Vp]
        s.set_lowrank(l, Up, Vp)
    Bp = torch.empty((nrhs, n_pad), dtype=torch.float64, device="cuda").t()
    hodlr.pad_rows(sizes, m_max, to_dev(B), Bp)
    torch.cuda.synchronize()
    s.factor()
    info = s.solve(Bp)
    X = torch.empty((nrhs, int(sizes.sum())), dtype=torch.float64, device="cuda").t()
    hodlr.unpad_rows(sizes, m_max, Bp, X)
    Xd = np.linalg.solve(A, B)
    x = to_host(X)
    assert np.linalg.norm(x - Xd) / np.linalg.norm(Xd) < (1e-11 if precision == 0 else 1e-10)
    # the padded rows of the solution stay exactly zero
    xp = to_host(Bp)
    for i, m in enumerate(sizes):
        assert np.abs(xp[i * m_max + m:(i + 1) * m_max]).max(initial=0.0) == 0.0
    if precision == 1:
        assert info.rel_residual <= 1e-12
    s.close()
