"""GPU tests of the component entry points, written after the reference's own
unit tests (tests/test.cc): gemm-reduce and gemm-broadcast (:316-372, two-level
variants :427-485), node solve with the swapped right-hand side (:374-425,
:487-541), the dense leaf blocks of the LMatrix init test (:245-258) and the
full HMatrix solve of test_solver (:544-661) through the C++ host library.
Tolerance: the reference's 1e-13 Frobenius norm for components."""
import json
import os
import subprocess

import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle import problems as P

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def dev(a):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        return torch.from_numpy(a.copy()).cuda()
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()


def host(t):
    return np.asfortranarray(t.t().cpu().numpy().T) if t.dim() == 2 else t.cpu().numpy()


def ld(t):
    return t.shape[0] if t.dim() == 1 or t.shape[1] == 1 else t.stride(1)


def rand(nPart, rows, cols, master):
    return O.rand_matrix(O.seeds(master, nPart), rows // nPart, cols)


@pytest.mark.parametrize("m,n,nPart", [(16, 3, 2), (16, 3, 4), (4096, 32, 8), (1 << 16, 16, 2)])
def test_gemm_reduce(hodlr, m, n, nPart):
    U = rand(nPart, m, n, 11)
    V = rand(nPart, m, n, 12)
    W = torch.zeros((n, nPart * n), dtype=torch.float64, device="cuda").t()
    Ud, Vd = dev(U), dev(V)
    hodlr.check(hodlr.lib().hodlr_gemm_reduce(m, nPart, n, n, Vd.data_ptr(), ld(Vd), Ud.data_ptr(), ld(Ud),
                                              W.data_ptr(), ld(W)))
    W = host(W)
    h = m // nPart
    for p in range(nPart):
        ref = V[p * h:(p + 1) * h].T @ U[p * h:(p + 1) * h]
        assert np.linalg.norm(W[p * n:(p + 1) * n] - ref) < 1e-13 * max(1.0, np.linalg.norm(ref))


@pytest.mark.parametrize("nPart,nBlock", [(8, 2), (8, 1), (4, 4)])
def test_gemm_broadcast(hodlr, nPart, nBlock):
    m, n = 16, 3
    U = rand(8, m, n, 21)
    Vb = rand(nBlock, nBlock * n, n, 22)
    W0 = rand(8, m, n, 23)
    Ud, Vd, Wd = dev(U), dev(Vb), dev(W0)
    for alpha, beta in ((1.0, 0.0), (-1.0, 1.0)):
        Wd = dev(W0)
        hodlr.check(hodlr.lib().hodlr_gemm_broadcast(m, nPart, nBlock, n, n, alpha, Ud.data_ptr(), ld(Ud),
                                                     Vd.data_ptr(), ld(Vd), beta, Wd.data_ptr(), ld(Wd)))
        ref = beta * W0.copy()
        rows, per = m // nPart, nPart // nBlock
        for p in range(nPart):
            blk = p // per
            ref[p * rows:(p + 1) * rows] += alpha * U[p * rows:(p + 1) * rows] @ Vb[blk * n:(blk + 1) * n]
        assert np.linalg.norm(host(Wd) - ref) < 1e-13


@pytest.mark.parametrize("nnode,r,nrhs", [(2, 3, 1), (4, 8, 5), (16, 32, 64)])
def test_node_solve(hodlr, nnode, r, nrhs):
    rng = np.random.default_rng(nnode * r)
    Vu = rng.random((nnode * 2 * r, r)) * (0.5 / r)   # keeps S well conditioned
    Vd = rng.random((nnode * 2 * r, nrhs))
    VTu, VTd = dev(Vu), dev(Vd)
    hodlr.check(hodlr.lib().hodlr_node_solve(nnode, r, nrhs, VTu.data_ptr(), ld(VTu), VTd.data_ptr(), ld(VTd)))
    out = host(VTd)
    for p in range(nnode):
        o = p * 2 * r
        S = np.eye(2 * r)
        S[r:, :r] = Vu[o:o + r]           # V0^T u0
        S[:r, r:] = Vu[o + r:o + 2 * r]   # V1^T u1
        rhs = np.vstack([Vd[o + r:o + 2 * r], Vd[o:o + r]])  # swapped halves
        sol = np.linalg.solve(S, rhs)
        assert np.linalg.norm(out[o:o + 2 * r] - sol) < 1e-13 * max(1.0, np.linalg.norm(sol))


def test_dense_blocks_and_uvd_solve(hodlr):
    m, L, r = 64, 3, 8
    pr = P.reference_problem(m, L, r, nrhs=1)
    nPart = 1 << L
    Dvec = O.rand_matrix(O.seeds(20240601 + 3, nPart), m, 1, offset=1000)[:, 0]
    s = hodlr.Solver(pr.n, m, L, r, nrhs_max=1)
    Ud, Vd, Dd = dev(pr.U[0]), dev(pr.V[0]), dev(Dvec)
    hodlr.check(hodlr.lib().hodlr_set_uvd(s.h, Ud.data_ptr(), ld(Ud), Vd.data_ptr(), ld(Vd), Dd.data_ptr()))
    K = torch.zeros((m, pr.n), dtype=torch.float64, device="cuda").t()
    s.get_inputs(D=K, ld=pr.n, leaf_stride=m)
    assert np.linalg.norm(host(K) - pr.K) < 1e-13 * np.linalg.norm(pr.K)
    B = dev(pr.B)
    s.factor()
    s.solve(B)
    Xo, _, _ = O.hsolve_general(pr, pr.B)
    assert np.linalg.norm(host(B) - Xo) / np.linalg.norm(Xo) < 1e-12


def _build_cpp(name="test_solver"):
    exe = os.path.join(ROOT, "tests", "cpp", name)
    src = os.path.join(ROOT, "tests", "cpp", name + ".cc")
    lib = os.path.join(ROOT, "fastsolver2_gb300")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(src):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                               "-I" + os.path.join(cuda, "include"), src, "-o", exe, "-L" + lib, "-lhodlr_gb300",
                               "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + lib])
    return exe


@pytest.mark.parametrize("leaf,levels,rank", [(64, 3, 8), (400, 2, 10), (128, 6, 16)])
def test_cpp_hmatrix_driver(hodlr, tmp_path, leaf, levels, rank):
    exe = _build_cpp()
    xfile = str(tmp_path / "x.bin")
    out = subprocess.run([exe, str(leaf), str(levels), str(rank), xfile], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    rep = json.loads(out.stdout.strip().splitlines()[-1])
    assert rep["rel_residual"] < 1e-12
    assert rep["seeded_rel_diff"] < 1e-12
    assert rep["checkpoint_identical"] is True
    x = np.fromfile(xfile, dtype=np.float64)
    pr = P.reference_problem(leaf, levels, rank, nrhs=1)
    Xo, _, _ = O.hsolve_general(pr, pr.B)
    assert np.linalg.norm(x - Xo[:, 0]) / np.linalg.norm(Xo) < 1e-12


def test_cpp_irregular_tree_driver(hodlr):
    """The C++ host class IrregularTree (and the unequal-rank LMatrix::node_solve)
    on a two-shard tree with a heavy shard and unequal ranks."""
    exe = _build_cpp("test_tree")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    rep = json.loads(out.stdout.strip().splitlines()[-1])
    assert rep["rows"] == (32 << 3) + (320 << 3)
    assert rep["rel_residual"] < 1e-12
    assert rep["node_solve_err"] < 1e-14
