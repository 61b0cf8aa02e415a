"""Checkpoint of a factored handle (hodlr_checkpoint_save / _load): a handle
loaded from the byte stream solves with the same bits as the handle that
wrote it, in both precision modes and for transposed solves; a damaged or
truncated stream is refused."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import problems as P
from tests.test_gpu_solver import make_solver, to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,resid", [(0, 0), (1, 2), (1, 1)])
@pytest.mark.parametrize("trans", [False, True])
def test_checkpoint_round_trip_gives_identical_solves(hodlr, precision, resid, trans):
    pr = P.gaussian_problem(128, 4, 32, nrhs=8, seed=31, orthonormal=True, decay=4.0, shift=1.5)
    s = make_solver(hodlr, pr, precision=precision, residual=resid, refine_tol=1e-12)
    s.set_tuning(red_ctas_per_sm=8, update_tile_rows=64, cap_warps=16, update_tc_shape=2, leaf_apply=1)
    s.factor()
    data = s.checkpoint()
    t = hodlr.Solver.from_checkpoint(data)
    assert (t.n, t.leaf, t.levels, t.rank) == (pr.n, pr.leaf, pr.levels, pr.rank)
    assert t.get_tuning()["red_ctas_per_sm"] == 8
    assert t.get_tuning()["cap_warps"] == 16 and t.get_tuning()["update_tc_shape"] == 2
    assert t.get_tuning()["leaf_apply"] == 1
    B0, B1 = to_dev(pr.B), to_dev(pr.B)
    i0 = s.solve(B0, transpose=trans)
    s.close()  # the loaded handle owns its own copies
    i1 = t.solve(B1, transpose=trans)
    np.testing.assert_array_equal(to_host(B0), to_host(B1))
    assert i0.iterations == i1.iterations
    assert i0.rel_residual == i1.rel_residual
    t.close()


def test_checkpoint_refuses_damage_and_unfactored_handles(hodlr):
    pr = P.gaussian_problem(64, 3, 8, nrhs=1, seed=3)
    s = make_solver(hodlr, pr)
    with pytest.raises(hodlr.HodlrError) as e:
        s.checkpoint()
    assert e.value.code == hodlr.HODLR_ERR_NOT_FACTORED
    s.factor()
    data = bytearray(s.checkpoint())
    h = ctypes.c_void_p()
    L = hodlr.lib()
    bad = bytearray(data)
    bad[len(bad) // 2] ^= 0x40  # one bit of the payload
    assert L.hodlr_checkpoint_load(bytes(bad), len(bad), None, ctypes.byref(h)) == hodlr.HODLR_ERR_INVALID_ARG
    assert b"checksum" in L.hodlr_last_error_string()
    short = bytes(data[:-8])
    assert L.hodlr_checkpoint_load(short, len(short), None, ctypes.byref(h)) == hodlr.HODLR_ERR_INVALID_ARG
    assert not h.value
    # an intact stream still loads after the refusals
    t = hodlr.Solver.from_checkpoint(bytes(data))
    B = to_dev(pr.B)
    t.solve(B)
    assert P.rel_residual(pr, to_host(B)) < 1e-10
    t.close()
    s.close()
