"""CPU tests of the C ABI library: it loads, exports exactly what
include/hodlr_gb300.h declares, and rejects bad arguments on the host
before touching a device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hodlr_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"HODLR_API\s+[\w\s\*]*?\b(hodlr_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def fs():
    import fastsolver2_gb300 as fs
    fs.lib(build_if_missing=True)
    return fs


def test_header_declares_api():
    names = declared_functions()
    for must in ["hodlr_hsolve", "hodlr_create", "hodlr_set_leaf_blocks", "hodlr_set_lowrank", "hodlr_factor",
                 "hodlr_solve", "hodlr_solve_transpose", "hodlr_adjoint", "hodlr_destroy",
                 "hodlr_last_error_string"]:
        assert must in names


def test_library_exports_every_declared_symbol(fs):
    L = fs.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
        assert name in fs.SIGNATURES, name


def test_bindings_cover_header(fs):
    assert set(fs.SIGNATURES) == set(declared_functions())


def test_hsolve_rejects_bad_partition(fs):
    L = fs.lib()
    buf = (ctypes.c_double * 64)()
    # nPart not a power of two
    assert L.hodlr_hsolve(12, 1, 1, 3, 12, buf, buf, buf) == fs.HODLR_ERR_INVALID_ARG
    # nrow not divisible by nPart
    assert L.hodlr_hsolve(10, 1, 1, 4, 10, buf, buf, buf) == fs.HODLR_ERR_INVALID_ARG
    # LD < nrow
    assert L.hodlr_hsolve(16, 1, 1, 2, 8, buf, buf, buf) == fs.HODLR_ERR_INVALID_ARG
    # rank out of range
    assert L.hodlr_hsolve(16, 1, 65, 2, 16, buf, buf, buf) == fs.HODLR_ERR_INVALID_ARG
    assert b"rank" in L.hodlr_last_error_string()


def test_create_rejects_bad_desc(fs):
    L = fs.lib()
    h = ctypes.c_void_p()
    bad = [
        fs.Desc(100, 10, 3, 4, 1, 0, 0, 1e-12, 10, 0, None),   # n != leaf * 2^levels
        fs.Desc(80, 10, 3, 0, 1, 0, 0, 1e-12, 10, 0, None),    # rank 0
        fs.Desc(80, 10, 3, 4, 0, 0, 0, 1e-12, 10, 0, None),    # nrhs_max 0
        fs.Desc(80, 10, 3, 4, 1, 7, 0, 1e-12, 10, 0, None),    # unknown precision
        fs.Desc(80, 10, 3, 4, 1, 1, 0, 0.0, 10, 0, None),      # mixed without tolerance
    ]
    for d in bad:
        assert L.hodlr_create(ctypes.byref(d), ctypes.byref(h)) == fs.HODLR_ERR_INVALID_ARG
        assert not h.value


def test_null_handle_calls_fail_cleanly(fs):
    L = fs.lib()
    assert L.hodlr_factor(None) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_solve(None, None, 0, 1, None) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_destroy(None) == fs.HODLR_OK
    t = fs.Tuning(4, 0, 8, 0, 0, -1.0)
    assert L.hodlr_set_tuning(None, t) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_autotune(None, 1, None) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_batch_autotune(None, None, 0) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_batch_factor(None) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_batch_destroy(None) == fs.HODLR_OK


def test_no_cpu_fallback_when_library_missing(monkeypatch, tmp_path):
    import fastsolver2_gb300 as fs
    monkeypatch.setattr(fs, "_lib", None)
    monkeypatch.setattr(fs, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(ImportError):
        fs.lib()


def test_checkpoint_load_rejects_bad_streams_on_host(fs):
    L = fs.lib()
    h = ctypes.c_void_p()
    # shorter than a header
    assert L.hodlr_checkpoint_load(b"HODLRCK1", 8, None, ctypes.byref(h)) == fs.HODLR_ERR_INVALID_ARG
    # a header-sized stream without the magic
    junk = bytes(256)
    assert L.hodlr_checkpoint_load(junk, len(junk), None, ctypes.byref(h)) == fs.HODLR_ERR_INVALID_ARG
    assert b"checkpoint" in L.hodlr_last_error_string()
    assert not h.value
    assert L.hodlr_checkpoint_size(None, None) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_checkpoint_save(None, None, 0) == fs.HODLR_ERR_INVALID_ARG


def test_draw_seeds_matches_glibc_lrand48_stream(fs):
    """hodlr_draw_seeds (host code) against the oracle's srand48_r/lrand48_r calls."""
    from oracle import oracle as O
    for master in (0, 1, 20240601, 2**31 - 1, 2**40 + 12345, -7):
        assert fs.draw_seeds(master, 37) == [int(x) for x in O.seeds(master, 37)]


def test_padding_calls_reject_bad_sizes_on_host(fs):
    L = fs.lib()
    buf = (ctypes.c_double * 16)()
    bad = (ctypes.c_int32 * 2)(3, 9)  # 9 > m_max
    assert L.hodlr_pad_rows(2, bad, 8, 1, buf, 16, buf, 16, None) == fs.HODLR_ERR_INVALID_ARG
    zero = (ctypes.c_int32 * 2)(0, 4)
    assert L.hodlr_unpad_rows(2, zero, 8, 1, buf, 16, buf, 16, None) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_pad_leaf_blocks(0, zero, 8, buf, buf, None) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_pad_leaf_blocks(2, bad, 8, None, buf, None) == fs.HODLR_ERR_INVALID_ARG


def test_wait_fault_hook_rejects_bad_arguments_on_host(fs):
    L = fs.lib()
    assert L.hodlr_debug_wait_fault(-2, 0, 0) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_debug_wait_fault(0, -1, 1000) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_debug_wait_fault(0, 0, -5) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_debug_wait_fault(0, 0, 2 * 10**9) == fs.HODLR_ERR_INVALID_ARG
    assert b"wait_fault" in L.hodlr_last_error_string()


def test_tree_calls_reject_bad_arguments_on_host(fs):
    """Argument checks of the irregular-tree entry points run before any device call."""
    L = fs.lib()
    d = fs.Desc(128, 32, 2, 4, 1, 0, 0, 1e-12, 10, 0, None)
    subs = (fs.Desc * 2)(d, d)
    h = ctypes.c_void_p()
    for top, ranks in ((0, [4, 4]), (8, [4, 4]), (1, [0, 4]), (1, [4, 65])):
        r = (ctypes.c_int32 * 2)(*ranks)
        desc = fs.TreeDesc(top, subs, r, 1, 0, None)
        assert L.hodlr_tree_create(ctypes.byref(desc), ctypes.byref(h)) == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_tree_create(None, ctypes.byref(h)) == fs.HODLR_ERR_INVALID_ARG
    for call in (lambda: L.hodlr_tree_factor(None), lambda: L.hodlr_tree_solve(None, None, 0, 1, None),
                 lambda: L.hodlr_tree_matvec(None, None, 0, None, 0, 1),
                 lambda: L.hodlr_tree_set_coupling(None, 0, 0, 0, None, 0, None, 0),
                 lambda: L.hodlr_tree_subtree(None, 0, ctypes.byref(h)),
                 lambda: L.hodlr_tree_rows(None, None, None)):
        assert call() == fs.HODLR_ERR_INVALID_ARG
    assert L.hodlr_tree_destroy(None) == fs.HODLR_OK
    bad = [(0, 4, 4, 1), (1, 0, 4, 1), (1, 4, 65, 1), (1, 4, 4, 0)]
    for nnode, r0, r1, k in bad:
        assert L.hodlr_node_solve_irregular(nnode, r0, r1, k, 8, 64, 8, 64, 8, 64, 8, 64) == fs.HODLR_ERR_INVALID_ARG
    # leading dimensions shorter than the stacked blocks
    assert L.hodlr_node_solve_irregular(2, 4, 3, 1, 8, 5, 8, 8, 8, 6, 8, 8) == fs.HODLR_ERR_INVALID_ARG
