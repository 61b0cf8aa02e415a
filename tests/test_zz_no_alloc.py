"""hodlr_gemm_reduce_noalloc -- the reduction for callers that cannot
allocate device memory -- checked against hodlr_gemm_reduce through the C ABI.

Callers under a framework allocator that owns the device, or in loops that
cannot absorb cudaMalloc's synchronisation, cannot call cudaMalloc; this entry
point takes its scratch from a fixed 16 MiB device array in the library
instead.  Two calls in a row with different shapes check that the shared
scratch carries nothing stale from one call into the next, and the device's
free memory is checked to stay put across calls.  This file sorts last so that
a stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _col(rows, cols, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn((cols, rows), dtype=torch.float64, device="cuda", generator=g).t()


def _call(fs, name, nrow, nPart, ncolV, ncolU, V, U):
    W = torch.full((ncolU, nPart * ncolV), float("nan"), dtype=torch.float64, device="cuda").t()
    f = getattr(fs.lib(), name)
    code = f(nrow, nPart, ncolV, ncolU, ctypes.c_void_p(V.data_ptr()), V.stride(1), ctypes.c_void_p(U.data_ptr()),
             U.stride(1), ctypes.c_void_p(W.data_ptr()), W.stride(1))
    return code, W


@pytest.mark.parametrize("first,second", [((1 << 16, 4, 32, 64), (4096, 2, 16, 5)),
                                          ((8192, 8, 8, 3), (1 << 17, 2, 64, 16))])
def test_noalloc_matches_allocating_entry_point(hodlr, first, second):
    for i, (nrow, nPart, ncolV, ncolU) in enumerate((first, second)):
        V, U = _col(nrow, ncolV, 10 + i), _col(nrow, ncolU, 20 + i)
        code, Wn = _call(hodlr, "hodlr_gemm_reduce_noalloc", nrow, nPart, ncolV, ncolU, V, U)
        assert code == hodlr.HODLR_OK, hodlr.lib().hodlr_last_error_string()
        code, Wr = _call(hodlr, "hodlr_gemm_reduce", nrow, nPart, ncolV, ncolU, V, U)
        assert code == hodlr.HODLR_OK
        a, b = Wn.cpu().numpy(), Wr.cpu().numpy()
        assert np.isfinite(a).all()
        np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-13 * np.abs(b).max())


def test_noalloc_allocates_no_device_memory(hodlr):
    """After the first call (which may load the library's device code, and
    with it the fixed array), further calls leave the device's free memory
    exactly where it was: cudaMalloc hands out whole pages, so any allocation
    would show."""
    nrow, nPart, ncolV, ncolU = 1 << 17, 8, 32, 64
    V, U = _col(nrow, ncolV, 3), _col(nrow, ncolU, 4)
    W = torch.zeros((ncolU, nPart * ncolV), dtype=torch.float64, device="cuda").t()
    f = hodlr.lib().hodlr_gemm_reduce_noalloc
    args = (nrow, nPart, ncolV, ncolU, ctypes.c_void_p(V.data_ptr()), V.stride(1), ctypes.c_void_p(U.data_ptr()),
            U.stride(1), ctypes.c_void_p(W.data_ptr()), W.stride(1))
    assert f(*args) == hodlr.HODLR_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert f(*args) == hodlr.HODLR_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_sizes_beyond_its_scratch(hodlr):
    nrow, nPart, ncolV, ncolU = 2048 * 32, 2048, 64, 64   # 2048*64*64 blocks > 2^21 doubles
    V, U = _col(nrow, ncolV, 1), _col(nrow, ncolU, 2)
    code, _ = _call(hodlr, "hodlr_gemm_reduce_noalloc", nrow, nPart, ncolV, ncolU, V, U)
    assert code == hodlr.HODLR_ERR_INVALID_ARG
    assert b"scratch" in hodlr.lib().hodlr_last_error_string()
