"""GPU parity tests: the CUDA path (through the C ABI) against the oracle.

Tolerances: leaf / capacitance factors 1e-13 relative (the reference's own
component tolerance, tests/test.cc:259-260); FP64 solutions 1e-12 relative and
relative residual <= 1e-10 (the FP64 parity bar); the mixed path must reach
its refinement target (1e-12).  Pivots must match bit for bit.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle import problems as P

pytestmark = pytest.mark.gpu


def to_dev(a):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        return torch.from_numpy(a.copy()).cuda()
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()


def to_host(t):
    if t.dim() == 1:
        return t.cpu().numpy()
    return np.asfortranarray(t.t().cpu().numpy().T)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def make_solver(fs, pr, nrhs=None, precision=0, **kw):
    s = fs.Solver(pr.n, pr.leaf, pr.levels, pr.rank, nrhs_max=nrhs or pr.nrhs, precision=precision, **kw)
    keep = [to_dev(pr.K)]
    s.set_leaf_blocks(keep[0])
    for l in range(pr.levels):
        U, V = to_dev(pr.U[l]), to_dev(pr.V[l])
        sv = to_dev(pr.s[l]) if pr.s is not None else None
        keep += [U, V, sv]
        s.set_lowrank(l, U, V, sv)
    torch.cuda.synchronize()
    return s


@pytest.mark.parametrize("m,L,r", [(64, 2, 8), (128, 3, 32), (256, 2, 16)])
def test_leaf_lu_matches_oracle(hodlr, m, L, r):
    pr = P.gaussian_problem(m, L, r, nrhs=1, seed=11)
    s = make_solver(hodlr, pr)
    s.factor()
    nleaf = 1 << L
    lu = torch.empty(nleaf * m * m, dtype=torch.float64, device="cuda")
    piv = torch.empty(pr.n, dtype=torch.int32, device="cuda")
    s.get_factors(leaf_lu=lu, leaf_ipiv=piv)
    lu = lu.cpu().numpy().reshape(nleaf, m, m)
    piv = piv.cpu().numpy().reshape(nleaf, m)
    for i in range(nleaf):
        LUo, pivo, info = O.dgetrf(pr.leaf_block(i))
        assert info == 0
        np.testing.assert_array_equal(piv[i], pivo)
        assert rel(lu[i].T, LUo) < 1e-13


@pytest.mark.parametrize("m,L,r,decay", [(32, 3, 4, None), (64, 4, 8, 6.0)])
def test_factors_match_oracle(hodlr, m, L, r, decay):
    pr = P.gaussian_problem(m, L, r, nrhs=1, seed=5, orthonormal=decay is not None, decay=decay,
                            shift=1.5 if decay else 4.0)
    s = make_solver(hodlr, pr)
    s.factor()
    X, f, info = O.hsolve_general(pr, pr.B, keep_factors=True)
    assert info == 0
    nnode = (1 << L) - 1
    ut = torch.empty((L * r, pr.n), dtype=torch.float64, device="cuda").t()
    cap = torch.empty(nnode * 4 * r * r, dtype=torch.float64, device="cuda")
    cpiv = torch.empty(nnode * 2 * r, dtype=torch.int32, device="cuda")
    s.get_factors(utilde=ut, cap_lu=cap, cap_ipiv=cpiv)
    ut = to_host(ut)
    for l in range(L):
        assert rel(ut[:, l * r:(l + 1) * r], f["utilde"][l]) < 1e-12
    cap = cap.cpu().numpy().reshape(nnode, 2 * r, 2 * r).transpose(0, 2, 1)
    np.testing.assert_array_equal(cpiv.cpu().numpy().reshape(nnode, 2 * r), f["cap_ipiv"])
    assert rel(cap, f["cap_lu"]) < 1e-12


@pytest.mark.parametrize("L,r", [(3, 32), (5, 8), (2, 40), (4, 24), (1, 3), (1, 40)])
def test_mixed_utilde_tensor_cores_match_fma_and_oracle(hodlr, L, r, monkeypatch):
    """Utilde = D^{-1} U of the mixed factorisation for 128-row leaves (U read
    in FP64): the tcgen05 kernel (exact three-way bf16 split, six partial
    products) against the FP32-FMA kernel on the same FP32 inverse -- equal
    to FP32 product rounding (a numpy emulation of both gives 2.4e-7) -- and
    both against the oracle's FP64 Utilde, to the FP32 inverse's accuracy.
    With one level the leaf application is all of Utilde; with more, the
    factorisation's FP32 updates of the ancestors' columns (also switched
    between tensor cores and FMA) add their own rounding.  Column counts L r
    that are not multiples of the 32-column tile included."""
    pr = P.gaussian_problem(128, L, r, nrhs=1, seed=23)
    _, f, info = O.hsolve_general(pr, pr.B, keep_factors=True)
    assert info == 0
    ref = np.concatenate([f["utilde"][l] for l in range(L)], axis=1)
    got = {}
    for tc in ("1", "0", "tuned-fma"):
        monkeypatch.setenv("HODLR_NO_TCGEN05", "1" if tc == "0" else "0")
        s = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED)
        if tc == "tuned-fma":  # the tuning knob: only the leaf application leaves the tensor cores
            s.set_tuning(leaf_apply=1)
            assert s.get_tuning()["leaf_apply"] == 1
        s.factor()
        ut = torch.empty((L * r, pr.n), dtype=torch.float64, device="cuda").t()
        s.get_factors(utilde=ut)
        got[tc] = to_host(ut)
    assert rel(got["1"], got["0"]) < (1e-6 if L == 1 else 1e-5)
    assert rel(got["1"], got["tuned-fma"]) < (1e-6 if L == 1 else 1e-5)
    if L == 1:  # no updates: the knob and the switch run the same FMA kernel
        assert np.array_equal(got["0"], got["tuned-fma"])
    for tc in got:
        assert rel(got[tc], ref) < 1e-4


@pytest.mark.parametrize("m,L,r", [(128, 4, 32), (64, 4, 20), (64, 3, 16), (32, 3, 5), (16, 2, 1)])
def test_mixed_capacitance_lu_matches_fp64(hodlr, m, L, r):
    # the mixed path factors S (assembled from FP32 reductions) in FP64 with
    # the same pivoting: same interchanges and factors within FP32 rounding
    # of S's entries; its FP32 inverse is checked through the solves below
    pr = P.gaussian_problem(m, L, r, nrhs=1, seed=21)
    nnode = (1 << L) - 1
    got = []
    for precision in (0, 1):
        s = make_solver(hodlr, pr, precision=precision)
        s.factor()
        cap = torch.empty(nnode * 4 * r * r, dtype=torch.float64, device="cuda")
        cpiv = torch.empty(nnode * 2 * r, dtype=torch.int32, device="cuda")
        s.get_factors(cap_lu=cap, cap_ipiv=cpiv)
        got.append((cap.cpu().numpy(), cpiv.cpu().numpy()))
        if precision == 1:
            B = to_dev(pr.B)
            info = s.solve(B)
            assert info.status == hodlr.HODLR_OK
            assert P.rel_residual(pr, to_host(B)) <= 1.5e-12
    np.testing.assert_array_equal(got[0][1], got[1][1])
    assert rel(got[1][0], got[0][0]) < 1e-4


@pytest.mark.parametrize("m,L,r,k", [(256, 4, 16, 1), (128, 5, 32, 8), (64, 6, 8, 3), (16, 0, 1, 2)])
def test_fp64_solve_matches_oracle(hodlr, m, L, r, k):
    pr = P.gaussian_problem(m, L, r, nrhs=k, seed=3)
    s = make_solver(hodlr, pr)
    s.factor()
    Xo, _, info = O.hsolve_general(pr, pr.B)
    B = to_dev(pr.B)
    info_gpu = s.solve(B)
    X = to_host(B)
    assert rel(X, Xo) < 1e-12
    assert P.rel_residual(pr, X) < 1e-10
    # a second solve replays the captured graph and must give the same bits
    B2 = to_dev(pr.B)
    s.solve(B2)
    assert torch.equal(B2, B) or np.array_equal(to_host(B2), X)


@pytest.mark.parametrize("name", ["ref_m16_L2_r3_k1", "ref_m64_L3_r8_k1", "ref_m32_L3_r4_k5",
                                  "ref_m256_L4_r16_k1", "ref_m400_L2_r10_k1"])
@pytest.mark.parametrize("where", ["device", "host"])
def test_hsolve_dropin_matches_golden(hodlr, name, where):
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    m, L, r, k = int(g["leaf"]), int(g["levels"]), int(g["rank"]), int(g["nrhs"])
    pr = P.reference_problem(m, L, r, nrhs=k, master=int(g["master"]), offset=int(g["offset"]))
    N = pr.n
    W = np.zeros((N, k + L * r), order="F")
    W[:, :k] = pr.B
    for l in range(L):
        W[:, k + l * r:k + (l + 1) * r] = pr.U[0]
    K = np.array(pr.K, order="F")
    V = np.array(pr.V[0], order="F")
    if where == "device":
        Kd, Wd, Vd = to_dev(K), to_dev(W), to_dev(V)
        hodlr.hsolve(N, k, r, 1 << L, N, Kd, Wd, Vd)
        K, W = to_host(Kd), to_host(Wd)
    else:
        hodlr.hsolve(N, k, r, 1 << L, N, K, W, V)
    assert rel(W[:, :k], g["x"]) < 1e-12
    if "region" in g:
        assert rel(W, g["region"]) < 1e-12
        assert rel(K, g["K"]) < 1e-12
    else:
        np.testing.assert_allclose(np.linalg.norm(W, axis=0), g["region_colnorms"], rtol=1e-12)
        assert rel(W[:64], g["region_head"]) < 1e-12
        assert rel(K[:64], g["K_head"]) < 1e-12


def test_hsolve_matches_restated_oracle_bigger(hodlr):
    pr = P.reference_problem(128, 6, 12, nrhs=2)
    N, L, r, k = pr.n, pr.levels, pr.rank, pr.nrhs
    W = np.zeros((N, k + L * r), order="F")
    W[:, :k] = pr.B
    for l in range(L):
        W[:, k + l * r:k + (l + 1) * r] = pr.U[0]
    K, V = np.array(pr.K, order="F"), np.array(pr.V[0], order="F")
    Wo, Ko = W.copy(order="F"), K.copy(order="F")
    assert O.hsolve(N, k, r, 1 << L, Ko, Wo, V) == 0
    hodlr.hsolve(N, k, r, 1 << L, N, K, W, V)
    assert rel(W, Wo) < 1e-12


@pytest.mark.parametrize("resid", [0, 1, 2])
def test_mixed_refinement_reaches_tolerance(hodlr, resid):
    pr = P.gaussian_problem(128, 6, 32, nrhs=4, seed=9, orthonormal=True, decay=6.0, shift=1.5)
    s = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, residual=resid, refine_tol=1e-12)
    s.factor()
    B = to_dev(pr.B)
    info = s.solve(B)
    X = to_host(B)
    assert info.rel_residual <= 1e-12
    assert info.iterations >= 1
    res = P.rel_residual(pr, X)
    assert res < 2e-12
    Xo, _, _ = O.hsolve_general(pr, pr.B)
    assert rel(X, Xo) < 1e-9


def _check_plu(A, lu, piv, tol):
    """P A = L U for one leaf: lu column-major (LAPACK layout), piv 1-based."""
    m = A.shape[0]
    Lf = np.tril(lu, -1) + np.eye(m)
    Uf = np.triu(lu)
    PA = np.array(A, copy=True)
    for i in range(m):
        p = piv[i] - 1
        PA[[i, p]] = PA[[p, i]]
    assert np.linalg.norm(PA - Lf @ Uf) / np.linalg.norm(A) < tol
    for k in range(m):  # partial pivoting: |L| <= 1
        assert np.abs(Lf[k + 1:, k]).max(initial=0.0) <= 1.0 + 1e-6


@pytest.mark.parametrize("transpose", [False, True])
def test_mixed_leaf128_inverse_and_factors_on_request(hodlr, transpose):
    """Leaf 128 in the mixed mode: the factorisation forms the FP32 leaf
    inverses by blocked Gauss-Jordan (no LU); solves refine to 1e-12 against
    a dense FP64 solve, forward and transposed; the leaf LU factors and
    pivots, asked for afterwards, are formed then and satisfy P A = L U."""
    pr = P.gaussian_problem(128, 3, 16, nrhs=3, seed=23, shift=1.5)
    s = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, refine_tol=1e-12)
    s.factor()
    B = to_dev(pr.B)
    info = s.solve(B, transpose=transpose)
    assert info.rel_residual <= 1e-12
    A = pr.dense()
    Xd = np.linalg.solve(A.T if transpose else A, pr.B)
    assert rel(to_host(B), Xd) < 1e-9
    nleaf = 1 << pr.levels
    lu = torch.empty(nleaf * 128 * 128, dtype=torch.float64, device="cuda")
    piv = torch.empty(pr.n, dtype=torch.int32, device="cuda")
    s.get_factors(leaf_lu=lu, leaf_ipiv=piv)
    lu = lu.cpu().numpy().reshape(nleaf, 128, 128)
    piv = piv.cpu().numpy().reshape(nleaf, 128)
    for i in range(nleaf):
        _check_plu(pr.leaf_block(i), lu[i].T, piv[i], 1e-5)


def test_mixed_hsolve_leaf128_writes_back_leaf_lu(hodlr):
    """The drop-in entry point in the mixed mode at leaf 128 leaves the leaf
    LU factors in K (dgesv's layout) as the FP64 path does: L U equals the
    leaf block up to a row permutation, in FP32 accuracy."""
    pr = P.reference_problem(128, 3, 8, nrhs=2, master=99)
    N, L, r, k = pr.n, pr.levels, pr.rank, pr.nrhs
    W = np.zeros((N, k + L * r), order="F")
    W[:, :k] = pr.B
    for l in range(L):
        W[:, k + l * r:k + (l + 1) * r] = pr.U[0]
    Kd, Wd, Vd = to_dev(pr.K), to_dev(W), to_dev(np.asfortranarray(pr.V[0]))
    info = hodlr.hsolve(N, k, r, 1 << L, N, Kd, Wd, Vd, precision=hodlr.PREC_MIXED)
    assert info.rel_residual <= 1e-12
    K = to_host(Kd)
    for i in range(1 << L):
        lu = K[i * 128:(i + 1) * 128]
        prod = (np.tril(lu, -1) + np.eye(128)) @ np.triu(lu)
        Pm = prod @ np.linalg.inv(pr.leaf_block(i))   # a permutation matrix, up to FP32 rounding
        Pr = np.rint(Pm)
        assert np.abs(Pm - Pr).max() < 1e-4
        assert (Pr.sum(axis=0) == 1).all() and (Pr.sum(axis=1) == 1).all() and (Pr >= 0).all()


def test_mixed_leaf128_singular_leaf_reported(hodlr):
    pr = P.gaussian_problem(128, 2, 8, nrhs=1, seed=4)
    pr.K[3 * 128:4 * 128, 5] = 0.0   # leaf 3: a zero column
    s = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED)
    with pytest.raises(hodlr.HodlrError) as e:
        s.factor()
    assert e.value.code == hodlr.HODLR_ERR_SINGULAR_LEAF
    assert "(index 3)" in str(e.value)


@pytest.mark.parametrize("precision", [0, 1])
def test_transpose_solve(hodlr, precision):
    pr = P.gaussian_problem(64, 4, 8, nrhs=3, seed=21, orthonormal=True, decay=3.0, shift=2.0)
    s = make_solver(hodlr, pr, precision=precision)
    s.factor()
    B = to_dev(pr.B)
    s.solve(B, transpose=True)
    Xd = np.linalg.solve(pr.dense().T, pr.B)
    assert rel(to_host(B), Xd) < 1e-11


def test_mixed_transpose_solve_follows_new_inputs(hodlr):
    """In the tensor-core residual mode the double-word copies that transposed
    solves use are made by the first transposed solve after the inputs change.
    A second problem set into the same handle (every leaf block and level)
    must be the one solved, before and after forward solves."""
    p1 = P.gaussian_problem(128, 5, 16, nrhs=2, seed=31, orthonormal=True, decay=3.0, shift=2.0)
    p2 = P.gaussian_problem(128, 5, 16, nrhs=2, seed=32, orthonormal=True, decay=3.0, shift=2.0)
    s = make_solver(hodlr, p1, precision=hodlr.PREC_MIXED, residual=hodlr.RESID_FP64_TENSOR, refine_tol=1e-12)
    for pr in (p1, p2):
        if pr is p2:
            keep = [to_dev(pr.K)]
            s.set_leaf_blocks(keep[0])
            for l in range(pr.levels):
                keep += [to_dev(pr.U[l]), to_dev(pr.V[l]), to_dev(pr.s[l])]
                s.set_lowrank(l, *keep[-3:])
            torch.cuda.synchronize()
        s.factor()
        for trans in (True, False, True):
            B = to_dev(pr.B)
            info = s.solve(B, transpose=trans)
            assert info.rel_residual <= 1e-12
            A = pr.dense()
            Xd = np.linalg.solve(A.T if trans else A, pr.B)
            assert rel(to_host(B), Xd) < 1e-11, (pr is p2, trans)


def _to_pinned(a):
    """A column-major copy in pinned host memory."""
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        return torch.from_numpy(a.copy()).pin_memory()
    return torch.from_numpy(np.ascontiguousarray(a.T)).pin_memory().t()


def test_set_from_pinned_host_matches_device_set(hodlr):
    """The mixed mode prepares the copies derived from each input on a side
    stream while the next input is copied.  Inputs set from pinned host memory
    -- one level first set to other values and overwritten straight away --
    solve to the same bits as the same inputs set from device memory."""
    pr = P.gaussian_problem(128, 5, 16, nrhs=3, seed=41, orthonormal=True, decay=3.0, shift=2.0)
    other = P.gaussian_problem(128, 5, 16, nrhs=3, seed=42, orthonormal=True, decay=3.0, shift=2.0)
    a = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, refine_tol=1e-12)
    b = hodlr.Solver(pr.n, pr.leaf, pr.levels, pr.rank, nrhs_max=pr.nrhs, precision=hodlr.PREC_MIXED,
                     refine_tol=1e-12)
    keep = [_to_pinned(pr.K)]
    b.set_leaf_blocks(keep[0])
    for l in range(pr.levels):
        if l == 2:
            keep += [_to_pinned(other.U[l]), _to_pinned(other.V[l]), _to_pinned(other.s[l])]
            b.set_lowrank(l, *keep[-3:])
        keep += [_to_pinned(pr.U[l]), _to_pinned(pr.V[l]), _to_pinned(pr.s[l])]
        b.set_lowrank(l, *keep[-3:])
    xs = []
    for s in (a, b):
        s.factor()
        B = to_dev(pr.B)
        torch.cuda.synchronize()
        info = s.solve(B)
        assert info.rel_residual <= 1e-12
        xs.append(to_host(B))
    assert np.array_equal(xs[0], xs[1])
    assert rel(xs[1], np.linalg.solve(pr.dense(), pr.B)) < 1e-11


@pytest.mark.parametrize("trans", [False, True])
def test_matvec_fp64(hodlr, trans):
    pr = P.gaussian_problem(64, 5, 8, nrhs=3, seed=4, orthonormal=True, decay=2.0)
    s = make_solver(hodlr, pr)
    X = to_dev(pr.B)
    Y = torch.zeros_like(X)
    Y = Y.t().contiguous().t()
    s.matvec(X, Y, transpose=trans)
    A = pr.dense()
    Yd = (A.T if trans else A) @ pr.B
    assert rel(to_host(Y), Yd) < 1e-13


def test_adjoint_matches_dense_gradient(hodlr):
    m, L, r, k = 64, 5, 6, 1
    pr = P.gaussian_problem(m, L, r, nrhs=k, seed=13, orthonormal=True, decay=2.0, shift=2.0)
    N = pr.n
    A = pr.dense()
    x = np.linalg.solve(A, pr.B)
    lam = np.linalg.solve(A.T, x)
    dA = -lam @ x.T
    s = make_solver(hodlr, pr)
    s.factor()
    xd, gd = to_dev(x), to_dev(x)
    db = torch.zeros((k, N), dtype=torch.float64, device="cuda").t()
    dD = torch.zeros((1 << L) * m * m, dtype=torch.float64, device="cuda")
    dU = torch.zeros(L * N * r, dtype=torch.float64, device="cuda")
    dV = torch.zeros(L * N * r, dtype=torch.float64, device="cuda")
    ds = torch.zeros(L * r, dtype=torch.float64, device="cuda")
    s.adjoint(xd, gd, db=db, dD=dD, dU=dU, dV=dV, ds=ds)
    assert rel(to_host(db), lam) < 1e-11
    dD = dD.cpu().numpy().reshape(1 << L, m, m).transpose(0, 2, 1)
    for i in range(1 << L):
        blk = dA[i * m:(i + 1) * m, i * m:(i + 1) * m]
        assert rel(dD[i], blk) < 1e-11
    dU = dU.cpu().numpy().reshape(L, r, N).transpose(0, 2, 1)
    dV = dV.cpu().numpy().reshape(L, r, N).transpose(0, 2, 1)
    ds = ds.cpu().numpy().reshape(L, r)
    for l in range(L):
        h = N >> (l + 1)
        sv = pr.s[l]
        gU = np.zeros((N, r))
        gV = np.zeros((N, r))
        gs = np.zeros(r)
        for p in range(1 << l):
            c0 = slice(2 * p * h, (2 * p + 1) * h)
            c1 = slice((2 * p + 1) * h, (2 * p + 2) * h)
            for a, b in ((c0, c1), (c1, c0)):
                blk = dA[a, b]
                gU[a] += (blk @ pr.V[l][b]) * sv
                gV[b] += (blk.T @ pr.U[l][a]) * sv
                gs += np.einsum("iq,ij,jq->q", pr.U[l][a], blk, pr.V[l][b])
        assert rel(dU[l], gU) < 1e-10
        assert rel(dV[l], gV) < 1e-10
        assert rel(ds[l], gs) < 1e-10


def test_generated_problem_solves(hodlr):
    m, L, r, k = 128, 7, 32, 4
    N = m << L
    s = hodlr.Solver(N, m, L, r, nrhs_max=k)
    B = torch.empty((k, N), dtype=torch.float64, device="cuda").t()
    s.generate(seed=7, shift=4.0, B=B)
    B0 = B.clone()
    s.factor()
    s.solve(B)
    R = torch.empty_like(B0).t().contiguous().t()
    s.matvec(B, R)
    res = torch.linalg.norm(R - B0) / torch.linalg.norm(B0)
    assert res.item() < 1e-12


@pytest.mark.parametrize("precision", [0, 1])
def test_singular_leaf_reports_status(hodlr, precision):
    """A zero leaf block is reported by the factorisation.  In the mixed mode
    the leaf LU starts on the handle's side stream when the leaf blocks are
    set, and the next factorisation takes over its status; a second
    factorisation runs its own leaf LU.  Good leaf blocks set afterwards
    factor and solve."""
    pr = P.gaussian_problem(32, 2, 4, nrhs=1, seed=2)
    good = pr.K.copy()
    pr.K[2 * 32:3 * 32, :] = 0.0  # leaf 2 all zeros
    s = make_solver(hodlr, pr, precision=precision)
    for _ in range(2):
        with pytest.raises(hodlr.HodlrError) as e:
            s.factor()
        assert e.value.code == hodlr.HODLR_ERR_SINGULAR_LEAF
    K = to_dev(good)
    s.set_leaf_blocks(K)
    torch.cuda.synchronize()
    s.factor()
    pr.K = good
    B = to_dev(pr.B)
    s.solve(B)
    assert rel(to_host(B), np.linalg.solve(pr.dense(), pr.B)) < 1e-11


def test_nonfinite_rhs_reports_status(hodlr):
    pr = P.gaussian_problem(32, 2, 4, nrhs=1, seed=2)
    s = make_solver(hodlr, pr)
    s.factor()
    B = pr.B.copy(order="F")
    B[17, 0] = np.nan
    Bd = to_dev(B)
    with pytest.raises(hodlr.HodlrError) as e:
        s.solve(Bd)
    assert e.value.code == hodlr.HODLR_ERR_NONFINITE_INPUT


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_picks_valid_shapes_and_keeps_results(hodlr, precision):
    pr = P.gaussian_problem(128, 6, 32, nrhs=4, seed=11, decay=2.0)
    s = make_solver(hodlr, pr, precision=precision)
    t = s.autotune(nrhs=4)
    assert t["red_ctas_per_sm"] in (2, 4, 8) and t["update_tile_rows"] in (0, 64) and t["ms"] > 0
    assert t["cap_warps"] in (0, 8, 16) and t["update_tc_shape"] in (0, 1, 2) and t["leaf_apply"] in (0, 1)
    got = s.get_tuning()
    assert all(got[key] == t[key]
               for key in ("red_ctas_per_sm", "update_tile_rows", "cap_warps", "update_tc_shape", "leaf_apply"))
    B = to_dev(pr.B)
    s.solve(B)   # autotune left the handle factored
    Xo, _, _ = O.hsolve_general(pr, pr.B)
    assert rel(to_host(B), Xo) < (1e-12 if precision == 0 else 1e-10)
    # every candidate shape gives the same solution up to rounding
    for red in (2, 8):
        for bm in (0, 64):
            s.set_tuning(red, bm)
            s.factor()
            B2 = to_dev(pr.B)
            s.solve(B2)
            assert rel(to_host(B2), Xo) < (1e-12 if precision == 0 else 1e-10)


@pytest.mark.parametrize("r", [16, 32, 48, 64])
def test_capacitance_and_update_shapes_keep_results(hodlr, r):
    """The mixed path's tuned kernel shapes (warps per capacitance system;
    tensor-core update tile and ring depth) change only rounding: each reaches
    the refinement target and agrees with the oracle's FP64 solve."""
    pr = P.gaussian_problem(128, 5, r, nrhs=5, seed=40 + r, orthonormal=True, decay=3.0, shift=1.5)
    s = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, refine_tol=1e-12)
    Xo, _, _ = O.hsolve_general(pr, pr.B)
    for warps in (0, 8, 16, 32):
        for shape in (0, 1, 2):
            s.set_tuning(cap_warps=warps, update_tc_shape=shape)
            assert s.get_tuning()["cap_warps"] == warps and s.get_tuning()["update_tc_shape"] == shape
            s.factor()
            B = to_dev(pr.B)
            info = s.solve(B)
            assert info.rel_residual <= 1e-12
            assert rel(to_host(B), Xo) < 1e-9
    with pytest.raises(hodlr.HodlrError):
        s.set_tuning(cap_warps=12)
    s.close()


@pytest.mark.parametrize("m,L,r,k", [(128, 6, 32, 4), (64, 5, 16, 3), (256, 3, 64, 2), (128, 4, 24, 70)])
def test_tensor_residual_matches_fp64_residual(hodlr, m, L, r, k):
    """The digit-product residual against a native FP64 residual of the same
    iterate: the refinement's reported residual must be the true one."""
    pr = P.gaussian_problem(m, L, r, nrhs=k, seed=21, orthonormal=True, decay=3.0, shift=1.5)
    s2 = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, residual=2, refine_tol=1e-12)
    s0 = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, residual=0, refine_tol=1e-12)
    s2.factor()
    s0.factor()
    B2, B0 = to_dev(pr.B), to_dev(pr.B)
    i2, i0 = s2.solve(B2), s0.solve(B0)
    X2 = to_host(B2)
    true = P.rel_residual(pr, X2)
    assert true < 2e-12
    assert abs(i2.rel_residual - i0.rel_residual) < 0.3 * max(i0.rel_residual, 1e-14) or true < 1e-13
    assert i2.iterations == i0.iterations


@pytest.mark.parametrize("m,L,r,k", [(128, 3, 32, 4), (256, 2, 16, 3), (128, 4, 24, 70), (128, 5, 8, 64),
                                     (256, 3, 64, 2), (128, 1, 40, 9)])
def test_tcgen05_residual_matches_mma_sync_residual(hodlr, m, L, r, k, monkeypatch):
    """The one-pass tcgen05 residual (leaf sizes 128 and 256) against the
    per-level mma.sync kernels on the same digits: same refinement path,
    residuals and solutions equal to FP64 refinement accuracy.  The switch
    also moves the FP32 update between the tensor cores and the FMA pipe, so
    the two final residuals belong to iterates that differ in FP32 rounding:
    they agree to the spread of that rounding (25 %), not to the last bit."""
    pr = P.gaussian_problem(m, L, r, nrhs=k, seed=33, orthonormal=True, decay=3.0, shift=1.5)
    out = {}
    for tc in ("0", "1"):
        monkeypatch.setenv("HODLR_NO_TCGEN05", "1" if tc == "0" else "0")
        s = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, residual=2, refine_tol=1e-12)
        s.factor()
        B = to_dev(pr.B)
        info = s.solve(B)
        out[tc] = (to_host(B), info.iterations, info.rel_residual)
    (X0, it0, r0), (X1, it1, r1) = out["0"], out["1"]
    assert it0 == it1
    assert abs(r1 - r0) <= 0.25 * max(r0, r1) + 1e-15, (r0, r1)
    assert max(r0, r1) <= 1e-12
    assert rel(X1, X0) < 1e-11
    assert P.rel_residual(pr, X1) < 2e-12


def test_tcgen05_residual_extreme_exponents(hodlr, monkeypatch):
    """Right-hand sides near the bottom of the FP32 range (B scaled by
    2^-80): the digit groups' scale factors leave the normal float range,
    which the tcgen05 epilogue handles on its ldexpf path; the scaled solve
    must match the unscaled one."""
    monkeypatch.setenv("HODLR_NO_TCGEN05", "0")
    pr = P.gaussian_problem(128, 3, 32, nrhs=4, seed=41, orthonormal=True, decay=3.0, shift=1.5)
    sc = 2.0 ** -80
    s = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, residual=2, refine_tol=1e-12)
    s.factor()
    B1, Bs = to_dev(pr.B), to_dev(pr.B * sc)
    i1, i2 = s.solve(B1), s.solve(Bs)
    X1, X2 = to_host(B1), to_host(Bs) / sc
    assert i2.status == hodlr.HODLR_OK and i2.rel_residual <= 1e-12
    assert rel(X2, X1) < 1e-11
    assert P.rel_residual(pr, X2) < 2e-12


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("rank0,rank1", [(12, 5), (3, 16)])
def test_unequal_sibling_ranks_by_zero_padding(hodlr, precision, rank0, rank1):
    """The irregular-rank tree of solver_irregular_ranks.cc / node_solve_region.cc:77-97
    (K01 = U0 V1^T with rank0 columns, K10 = U1 V0^T with rank1) solved by the uniform
    path with bases zero-padded to max(rank0, rank1)."""
    m, L = 64, 4
    r = max(rank0, rank1)
    pr = P.gaussian_problem(m, L, r, nrhs=3, seed=44, orthonormal=True, decay=2.0, shift=2.0)
    for l in range(L):
        half = pr.n >> (l + 1)
        for c in range(2 << l):
            rows = slice(c * half, (c + 1) * half)
            ru, rv = (rank0, rank1) if c % 2 == 0 else (rank1, rank0)
            pr.U[l][rows, ru:] = 0.0
            pr.V[l][rows, rv:] = 0.0
    s = make_solver(hodlr, pr, precision=precision, refine_tol=1e-12)
    s.factor()
    B = to_dev(pr.B)
    info = s.solve(B)
    X = to_host(B)
    Xd = np.linalg.solve(pr.dense(), pr.B)
    assert rel(X, Xd) < (1e-11 if precision == 0 else 1e-10)
    if precision == 1:
        assert info.rel_residual <= 1e-12


@pytest.mark.parametrize("resid", [0, 1, 2])
def test_refinement_loop_same_eager_captured_replayed(hodlr, resid):
    """The first solve runs the refinement loop unrolled and predicated; the
    second captures it as a graph conditional WHILE node, the third replays
    it.  An unreachable tolerance makes the loop run all refine_max_iter
    corrections and stop with HODLR_ERR_NOT_CONVERGED every time, leaving
    the same iterate; a reachable one gives bitwise-equal solutions."""
    pr = P.gaussian_problem(128, 5, 32, nrhs=3, seed=5, orthonormal=True, decay=6.0, shift=1.5)
    s = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, residual=resid, refine_tol=1e-30, refine_max_iter=3)
    s.factor()
    B0 = to_dev(pr.B)
    B = to_dev(pr.B)   # one buffer: solve graphs are cached per right-hand-side pointer
    outs = []
    for _ in range(3):
        B.copy_(B0)
        torch.cuda.synchronize()   # the library runs on its own stream
        with pytest.raises(hodlr.HodlrError) as e:
            s.solve(B)
        assert e.value.code == hodlr.HODLR_ERR_NOT_CONVERGED
        assert "after 3 corrections" in str(e.value)
        outs.append(to_host(B))
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])
    s.close()
    s = make_solver(hodlr, pr, precision=hodlr.PREC_MIXED, residual=resid, refine_tol=1e-12, refine_max_iter=10)
    s.factor()
    outs, its = [], []
    for _ in range(3):
        B.copy_(B0)
        torch.cuda.synchronize()   # the library runs on its own stream
        info = s.solve(B)
        assert info.rel_residual <= 1e-12
        outs.append(to_host(B))
        its.append(info.iterations)
    assert its[0] == its[1] == its[2] >= 1
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])
    s.close()


def _pinned_colmajor(a):
    """A pinned host tensor holding the Fortran-ordered array a, column-major."""
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).pin_memory().t()


@pytest.mark.parametrize("precision", [0, 1])
def test_streamed_v_inputs_match_plain_inputs(hodlr, precision):
    """HODLR_FLAG_STREAM_INPUTS: V from pinned host memory is copied by the
    factorisation (deepest level first, beside the sweep).  Factor + solve in
    the eager, captured and replayed runs, and again after the host buffers
    change (the streamed graphs are captured again), equal a handle whose
    inputs were set from the device, bit for bit; a product before any
    factorisation copies the waiting V first."""
    pr = P.gaussian_problem(128, 5, 32, nrhs=4, seed=77, orthonormal=True, decay=3.0, shift=1.5)
    ref = make_solver(hodlr, pr, precision=precision, refine_tol=1e-12)
    ref.factor()
    Bref = to_dev(pr.B)
    ref.solve(Bref)
    xref = to_host(Bref)
    X = to_dev(np.random.default_rng(3).standard_normal((pr.n, 4)))
    Yref = torch.empty((4, pr.n), dtype=torch.float64, device="cuda").t()
    ref.matvec(X, Yref)
    torch.cuda.synchronize()

    s = hodlr.Solver(pr.n, pr.leaf, pr.levels, pr.rank, nrhs_max=4, precision=precision, refine_tol=1e-12,
                     flags=hodlr.FLAG_STREAM_INPUTS)
    D = to_dev(pr.K)
    s.set_leaf_blocks(D)
    sets = [[(_pinned_colmajor(pr.U[l]), _pinned_colmajor(pr.V[l])) for l in range(pr.levels)] for _ in range(2)]
    sv = [to_dev(pr.s[l]) for l in range(pr.levels)] if pr.s is not None else [None] * pr.levels

    def set_all(which):
        for l in range(pr.levels):
            s.set_lowrank(l, sets[which][l][0], sets[which][l][1], sv[l])

    set_all(0)
    Y = torch.empty((4, pr.n), dtype=torch.float64, device="cuda").t()
    s.matvec(X, Y)                      # before any factorisation: the waiting V is copied first
    torch.cuda.synchronize()
    assert torch.equal(Y, Yref)
    B = to_dev(pr.B)
    for which in (0, 0, 0, 1, 1):       # eager, captured, replayed; new buffers: captured, replayed
        set_all(which)
        s.factor()
        B.copy_(to_dev(pr.B))
        torch.cuda.synchronize()
        s.solve(B)
        np.testing.assert_array_equal(to_host(B), xref)
    s.close()
    ref.close()
