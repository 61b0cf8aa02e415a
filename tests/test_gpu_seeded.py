"""The reference's seeded generator on the device (hodlr_rand_matrix,
hodlr_set_seeded) against the oracle's drand48 restatement, bit for bit at
oracle sizes and by spot checks of single leaves at N = 2^20; the problems of
the golden fixtures, built on the device, solve to the verbatim reference
build's solutions."""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle import problems as P
from tests.test_gpu_solver import to_host

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("npart,rows,cols,offset", [(1, 5, 3, 0.0), (8, 64, 16, 0.0), (16, 128, 1, 1000.0),
                                                    (4, 400, 10, 0.0), (3, 33, 7, -2.5)])
def test_rand_matrix_is_bit_identical(hodlr, npart, rows, cols, offset):
    seeds = O.seeds(1234 + npart, npart)
    A = torch.full((cols, npart * rows + 3), np.nan, dtype=torch.float64, device="cuda").t()  # ld > rows
    hodlr.rand_matrix(seeds, rows, A[: npart * rows], offset=offset)
    ref = O.rand_matrix(seeds, rows, cols, offset=0)
    if offset:
        ref = ref + offset  # the oracle adds an integer offset the same way
    got = to_host(A)[: npart * rows]
    np.testing.assert_array_equal(got.view(np.uint64), np.asarray(ref, order="F").view(np.uint64))
    assert np.isnan(to_host(A)[npart * rows:]).all()  # rows past the partitions untouched


@pytest.mark.parametrize("name", ["ref_m16_L2_r3_k1", "ref_m64_L3_r8_k1", "ref_m32_L3_r4_k5",
                                  "ref_m256_L4_r16_k1", "ref_m400_L2_r10_k1"])
def test_seeded_inputs_match_golden_and_solve(hodlr, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    m, L, r, k, master = int(g["leaf"]), int(g["levels"]), int(g["rank"]), int(g["nrhs"]), int(g["master"])
    nP = 1 << L
    n = m * nP
    vs, us, bs, ds = (hodlr.draw_seeds(master + i, nP) for i in range(4))
    s = hodlr.Solver(n, m, L, r, nrhs_max=k)
    s.set_seeded(us, vs, ds, offset=float(g["offset"]))
    D = torch.empty(nP * m * m, dtype=torch.float64, device="cuda")
    U = torch.empty((L * r, n), dtype=torch.float64, device="cuda").t()
    V = torch.empty((L * r, n), dtype=torch.float64, device="cuda").t()
    sv = torch.empty(L * r, dtype=torch.float64, device="cuda")
    s.get_inputs(D=D, ld=m, leaf_stride=m * m, U=U, V=V, s=sv)
    pr = P.reference_problem(m, L, r, nrhs=k, master=master)
    K = D.cpu().numpy().reshape(nP, m, m).transpose(0, 2, 1).reshape(n, m)  # KTree layout: leaf i at rows i*m
    np.testing.assert_array_equal(K.view(np.uint64), np.ascontiguousarray(pr.K).view(np.uint64))
    Uh, Vh = to_host(U), to_host(V)
    for l in range(L):
        np.testing.assert_array_equal(Uh[:, l * r:(l + 1) * r], pr.U[0])
        np.testing.assert_array_equal(Vh[:, l * r:(l + 1) * r], pr.V[0])
    assert (sv.cpu().numpy() == 1.0).all()
    B = torch.empty((k, n), dtype=torch.float64, device="cuda").t()
    hodlr.rand_matrix(bs, m, B)
    np.testing.assert_array_equal(to_host(B), pr.B)
    s.factor()
    s.solve(B)
    x = to_host(B)
    assert np.linalg.norm(x - g["x"]) / np.linalg.norm(g["x"]) < 1e-12
    s.close()


def test_seeded_inputs_at_full_size_spot_checks(hodlr):
    """N = 2^20, leaf 128, 13 levels, rank 32: leaves 0, 4097 and 8191 of the
    device-built problem against the oracle's generator for those leaves."""
    m, L, r = 128, 13, 32
    nP = 1 << L
    n = m * nP
    vs, us, ds = (hodlr.draw_seeds(77 + i, nP) for i in range(3))
    s = hodlr.Solver(n, m, L, r)
    s.set_seeded(us, vs, ds, offset=1000.0)
    D = torch.empty(nP * m * m, dtype=torch.float64, device="cuda")
    U = torch.empty((L * r, n), dtype=torch.float64, device="cuda").t()
    s.get_inputs(D=D, ld=m, leaf_stride=m * m, U=U)
    Dh = D.view(nP, m, m)
    for leaf in (0, 4097, nP - 1):
        blk = O.dense_blocks([us[leaf]], [vs[leaf]], [ds[leaf]], m, r, 1000)
        got = Dh[leaf].cpu().numpy().T  # stored column-major
        np.testing.assert_array_equal(got.view(np.uint64), np.ascontiguousarray(blk).view(np.uint64))
        u = O.rand_matrix([us[leaf]], m, r)
        for l in (0, 7, L - 1):
            np.testing.assert_array_equal(U[leaf * m:(leaf + 1) * m, l * r:(l + 1) * r].cpu().numpy(), u)
    s.close()
