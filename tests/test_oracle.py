"""CPU tests of the oracle: pinned against the reference's own hsolve (golden
fixtures produced by the verbatim build, and the build itself where the
reference checkout is mounted), against dense LAPACK, and for internal
consistency (restated netlib LU, multithreaded baseline, matvec)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle import problems as P

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def ref_region(pr):
    N, L, r, k = pr.n, pr.levels, pr.rank, pr.nrhs
    W = np.zeros((N, k + L * r), order="F")
    W[:, :k] = pr.B
    for l in range(L):
        W[:, k + l * r:k + (l + 1) * r] = pr.U[0]
    return W


def test_golden_fixtures_present():
    assert len(CASES) >= 5


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_golden(oracle_lib, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    m, L, r, k = int(g["leaf"]), int(g["levels"]), int(g["rank"]), int(g["nrhs"])
    pr = P.reference_problem(m, L, r, nrhs=k, master=int(g["master"]), offset=int(g["offset"]))
    K = np.array(pr.K, order="F")
    W = ref_region(pr)
    V = np.array(pr.V[0], order="F")
    assert O.hsolve(pr.n, k, r, 1 << L, K, W, V) == 0
    assert rel(W[:, :k], g["x"]) < 1e-13
    if "region" in g:
        assert rel(W, g["region"]) < 1e-13
        assert rel(K, g["K"]) < 1e-13
    else:
        np.testing.assert_allclose(np.linalg.norm(W, axis=0), g["region_colnorms"], rtol=1e-13)
        assert rel(W[:64], g["region_head"]) < 1e-13
        assert rel(K[:64], g["K_head"]) < 1e-13
    # the generalised recursion, given the shared U / V, is the same computation
    X, _, info = O.hsolve_general(pr, pr.B)
    assert info == 0
    assert rel(X, g["x"]) < 1e-13


def test_generator_matches_reference_fill_order(oracle_lib):
    # PtrMatrix::rand fills a column-major block in row-major order
    # (src/ptr_matrix.cc:62-71): consecutive drand48 draws run along a row.
    seed = 12345
    A = np.zeros((3, 4), order="F")
    O.lib().orc_rand_block(seed, 3, 4, 3, O._p(A), 0)
    flat = np.zeros((1, 12), order="F")
    O.lib().orc_rand_block(seed, 1, 12, 1, O._p(flat), 0)
    np.testing.assert_array_equal(A.reshape(-1), flat.reshape(-1))
    assert (A >= 0).all() and (A < 1).all()


@pytest.mark.parametrize("name", CASES[:3])
def test_verbatim_reference_matches_oracle(oracle_lib, name):
    if O.ref_lib() is None:
        pytest.skip("reference checkout not mounted here")
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    m, L, r, k = int(g["leaf"]), int(g["levels"]), int(g["rank"]), int(g["nrhs"])
    pr = P.reference_problem(m, L, r, nrhs=k, master=int(g["master"]))
    K, W, V = np.array(pr.K, order="F"), ref_region(pr), np.array(pr.V[0], order="F")
    O.ref_hsolve(pr.n, k, r, 1 << L, K, W, V)
    assert rel(W[:, :k], g["x"]) < 1e-15  # fixtures came from this build


@pytest.mark.parametrize("n", [1, 7, 64, 130, 256])
def test_dgetrf_pivots_match_lapack(oracle_lib, n):
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    LU, piv, info = O.dgetrf(A)
    assert info == 0
    lu_s, piv_s = scipy_linalg.lu_factor(A)
    np.testing.assert_array_equal(piv, piv_s + 1)
    assert rel(LU, lu_s) < 1e-13


def test_dgetrf_singular_info(oracle_lib):
    A = np.ones((5, 5))
    _, _, info = O.dgetrf(A)
    assert info == 2


def test_dgetrs_both_transposes(oracle_lib):
    rng = np.random.default_rng(1)
    A = rng.standard_normal((40, 40)) + 5 * np.eye(40)
    B = rng.standard_normal((40, 3))
    LU, piv, _ = O.dgetrf(A)
    assert rel(O.dgetrs(LU, piv, B, "N"), np.linalg.solve(A, B)) < 1e-13
    assert rel(O.dgetrs(LU, piv, B, "T"), np.linalg.solve(A.T, B)) < 1e-13


@pytest.mark.parametrize("kw", [dict(), dict(orthonormal=True, decay=6.0, shift=1.5)])
def test_general_solve_matches_dense(oracle_lib, kw):
    pr = P.gaussian_problem(32, 4, 6, nrhs=3, seed=2, **kw)
    X, f, info = O.hsolve_general(pr, pr.B, keep_factors=True)
    assert info == 0
    Xd = np.linalg.solve(pr.dense(), pr.B)
    assert rel(X, Xd) < 1e-12
    assert P.rel_residual(pr, X) < 1e-14
    # stored leaf factors reproduce the leaf blocks
    for i in range(1 << pr.levels):
        LU = f["leaf_lu"][i * 32:(i + 1) * 32]
        np.testing.assert_array_equal(f["leaf_ipiv"][i], O.dgetrf(pr.leaf_block(i))[1])
        assert rel(LU, O.dgetrf(pr.leaf_block(i))[0]) == 0.0


@pytest.mark.parametrize("threads", [2, 4, 8])
def test_threaded_baseline_matches_serial(oracle_lib, threads):
    pr = P.gaussian_problem(32, 5, 4, nrhs=2, seed=8, decay=1.0)
    X1, _, _ = O.hsolve_general(pr, pr.B)
    Xt, _, info = O.hsolve_general(pr, pr.B, nthreads=threads)
    assert info == 0
    assert rel(Xt, X1) < 1e-13


def test_hodlr_matvec_matches_dense(oracle_lib):
    pr = P.gaussian_problem(16, 4, 3, nrhs=2, seed=5, orthonormal=True, decay=3.0)
    np.testing.assert_allclose(O.hodlr_matvec(pr, pr.B), pr.dense() @ pr.B, rtol=0, atol=1e-13)


def test_singular_leaf_detected(oracle_lib):
    pr = P.gaussian_problem(16, 2, 2, nrhs=1, seed=1)
    pr.K[16:32] = 0.0
    _, _, info = O.hsolve_general(pr, pr.B)
    assert info == 2  # leaf 1, reported as 1 + leaf index


def test_edge_single_leaf(oracle_lib):
    pr = P.gaussian_problem(24, 0, 1, nrhs=2, seed=1)
    X, _, info = O.hsolve_general(pr, pr.B)
    assert info == 0
    assert rel(X, np.linalg.solve(pr.K, pr.B)) < 1e-13


# ------------------------------------------------ the BLAS-backed restatement
def _need_blas():
    if O.blas_lib() is None:
        pytest.skip("scipy's OpenBLAS not available")


@pytest.mark.parametrize("name", CASES)
def test_blas_hsolve_matches_golden(oracle_lib, name):
    """hsolve with its dgemm_/dgesv_ calls on OpenBLAS (the CPU baseline's
    arithmetic) reproduces the fixtures of the verbatim reference build."""
    _need_blas()
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    m, L, r, k = int(g["leaf"]), int(g["levels"]), int(g["rank"]), int(g["nrhs"])
    pr = P.reference_problem(m, L, r, nrhs=k, master=int(g["master"]), offset=int(g["offset"]))
    K, W, V = np.array(pr.K, order="F"), ref_region(pr), np.array(pr.V[0], order="F")
    assert O.blas_hsolve(pr.n, k, r, 1 << L, K, W, V) == 0
    assert rel(W[:, :k], g["x"]) < 1e-13


@pytest.mark.parametrize("m,L,r,k", [(16, 2, 3, 1), (64, 3, 8, 1), (32, 4, 4, 5), (128, 4, 16, 3)])
def test_blas_hsolve_is_bitwise_the_verbatim_reference(oracle_lib, m, L, r, k):
    """Same calls in the same order on the same BLAS: the same bits as the
    reference's own hsolve compiled against that BLAS."""
    _need_blas()
    if O.ref_lib() is None:
        pytest.skip("reference checkout not mounted here")
    pr = P.reference_problem(m, L, r, nrhs=k, master=777 + m)
    K1, W1, V = np.array(pr.K, order="F"), ref_region(pr), np.array(pr.V[0], order="F")
    K2, W2 = K1.copy(order="F"), W1.copy(order="F")
    O.ref_hsolve(pr.n, k, r, 1 << L, K1, W1, V)
    assert O.blas_hsolve(pr.n, k, r, 1 << L, K2, W2, V) == 0
    np.testing.assert_array_equal(W1, W2)
    np.testing.assert_array_equal(K1, K2)


@pytest.mark.parametrize("nthreads", [1, 2, 8])
def test_blas_hsolve_mt_matches_oracle(oracle_lib, nthreads):
    """The threaded baseline (subtrees per thread, then row-chunked top
    levels) against the oracle's generalised recursion, per-level factors."""
    _need_blas()
    pr = P.gaussian_problem(32, 5, 6, nrhs=3, seed=5)
    X0, _, info = O.hsolve_general(pr, pr.B)
    assert info == 0
    L, r, k = pr.levels, pr.rank, pr.nrhs
    K = np.array(pr.K, order="F")
    W = np.zeros((pr.n, k + L * r), order="F")
    W[:, :k] = pr.B
    for l in range(L):
        W[:, k + l * r:k + (l + 1) * r] = pr.U[l]
    Vs = [np.asfortranarray(v) for v in pr.V]
    assert O.blas_hsolve_mt(pr.leaf, L, r, K, Vs, W, k, nthreads) == 0
    assert rel(W[:, :k], X0) < 1e-12


@pytest.mark.parametrize("nthreads", [1, 4, 16])
def test_blas_matvec_matches_oracle(oracle_lib, nthreads):
    _need_blas()
    pr = P.gaussian_problem(16, 5, 4, nrhs=3, seed=9, decay=2.0)
    Y0 = O.hodlr_matvec(pr, pr.B)
    Y = O.blas_matvec(pr.leaf, pr.levels, pr.rank, np.asfortranarray(pr.K), pr.U, pr.V, pr.s,
                      np.asfortranarray(pr.B), nthreads)
    assert rel(Y, Y0) < 1e-13


@pytest.mark.parametrize("r0,r1,k", [(5, 3, 2), (1, 7, 1), (12, 12, 4)])
def test_node_solve_irregular_oracle_matches_dense(oracle_lib, r0, r1, k):
    """node_solve_region.cc:77-97: [I, VTu1; VTu0, I] [eta0; eta1] = [VTd1; VTd0],
    eta0 written to VTd1 and eta1 to VTd0."""
    rng = np.random.default_rng(r0 * 31 + r1)
    VTu0, VTu1 = rng.standard_normal((r1, r0)) * 0.3, rng.standard_normal((r0, r1)) * 0.3
    VTd0, VTd1 = rng.standard_normal((r1, k)), rng.standard_normal((r0, k))
    o0, o1, info = O.node_solve_irregular(r0, r1, VTu0, VTu1, VTd0, VTd1)
    S = np.block([[np.eye(r0), VTu1], [VTu0, np.eye(r1)]])
    eta = np.linalg.solve(S, np.vstack([VTd1, VTd0]))
    assert info == 0
    assert rel(o1, eta[:r0]) < 1e-14 and rel(o0, eta[r0:]) < 1e-14


@pytest.mark.parametrize("T,shapes,ranks", [
    (1, [(16, 2, 3), (160, 2, 3)], [3, 3]),                                    # heavy shard, leaf x10
    (1, [(32, 2, 6), (32, 2, 2)], [6, 2]),                                     # shard ranks rank0 / rank1
    (2, [(16, 2, 3), (160, 2, 3), (16, 3, 5), (32, 1, 2)], [5, 3, 4, 6, 2, 7]),
])
def test_tree_oracle_matches_dense(oracle_lib, T, shapes, ranks):
    tp = P.tree_problem(T, shapes, ranks, nrhs=3, seed=T + len(shapes))
    X, info = O.tree_solve(tp, tp.B)
    A = tp.dense()
    assert info == 0
    assert rel(X, np.linalg.solve(A, tp.B)) < 1e-13
    assert rel(tp.matvec(X), A @ X) < 1e-14
