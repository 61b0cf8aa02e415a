"""The exact three-way bf16 split and the six partial products that the
tcgen05 kernels (the low-rank update, the row reductions and the leaf
application) use for FP32-class products, restated in numpy:

* split3_pair / put_planes (fastsolver2_gb300/csrc/tcgen05.cuh): every FP32
  value x is h + m + l exactly, h = bf16(x), m = bf16(x - h), l = bf16(x - h - m);
* the products keep hh, hm + mh and hl + mm + lh (the leaf application's three
  N-concatenated accumulator groups) and drop ml, lm, ll, which together stay
  below 2^-23 of |a| |b| per product;
* a 128-term dot product formed that way is as close to the exact one as the
  FP32 FMA dot product the FMA kernels form (the leaf application's K = 128).
"""
import numpy as np


def bf16_rn(x):
    """Round FP32 values to bf16 (nearest, ties to even), returned as FP32."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def split3(x):
    x = np.asarray(x, dtype=np.float32)
    h = bf16_rn(x)
    r1 = (x - h).astype(np.float32)
    m = bf16_rn(r1)
    l = bf16_rn((r1 - m).astype(np.float32))
    return h, m, l


def test_split_is_exact():
    rng = np.random.default_rng(3)
    x = (rng.standard_normal(1 << 18) * 10.0 ** rng.uniform(-20, 20, 1 << 18)).astype(np.float32)
    h, m, l = split3(x)
    # the three parts sum back to x exactly (in FP64, where the sum cannot round)
    assert np.array_equal(h.astype(np.float64) + m.astype(np.float64) + l.astype(np.float64), x.astype(np.float64))
    # each part is a bf16 value
    for p in (h, m, l):
        assert np.array_equal(bf16_rn(p), p)


def test_dropped_products_below_fp32_rounding():
    rng = np.random.default_rng(4)
    a = rng.standard_normal(1 << 18).astype(np.float32)
    b = rng.standard_normal(1 << 18).astype(np.float32)
    ah, am, al = (p.astype(np.float64) for p in split3(a))
    bh, bm, bl = (p.astype(np.float64) for p in split3(b))
    kept = ah * bh + (ah * bm + am * bh) + (ah * bl + am * bm + al * bh)
    exact = a.astype(np.float64) * b.astype(np.float64)
    rel = np.abs(kept - exact) / np.abs(exact)
    assert rel.max() < 2.0 ** -23


def test_grouped_dot_products_match_fp32_class():
    """K = 128 dot products as the leaf application forms them: three groups
    accumulated in FP32 (the tensor-memory accumulator), summed smallest
    first; against the exact FP64 product and against an FP32 multiply-add
    chain (each product and each sum rounded to FP32)."""
    rng = np.random.default_rng(5)
    K, M, N = 128, 64, 64
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    Ah, Am, Al = split3(A)
    Bh, Bm, Bl = split3(B)
    f = lambda x, y: (x.astype(np.float32) @ y.astype(np.float32)).astype(np.float32)
    g0 = f(Ah, Bh)
    g1 = (f(Ah, Bm) + f(Am, Bh)).astype(np.float32)
    g2 = (f(Ah, Bl) + f(Am, Bm) + f(Al, Bh)).astype(np.float32)
    tc = ((g2 + g1).astype(np.float32) + g0).astype(np.float32)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    fma = np.zeros((M, N), dtype=np.float32)
    for k in range(K):  # FP32 rounding of each product and each sum
        fma = (fma + np.outer(A[:, k], B[k, :]).astype(np.float32)).astype(np.float32)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    err_tc = np.max(np.abs(tc - exact) / scale)
    err_fma = np.max(np.abs(fma - exact) / scale)
    assert err_tc < 8 * 2.0 ** -24 * np.sqrt(K)
    assert err_tc < 2 * err_fma + 2.0 ** -23
