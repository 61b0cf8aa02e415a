"""The FP64 -> FP32 conversion the staging kernels run on the integer pipes
(`f64_to_f32_rn`, fastsolver2_gb300/csrc/common.cuh), restated step for step
in numpy on the same 32-bit words, against numpy's own round-to-nearest-even
cast: bit for bit over random magnitudes across the whole double range,
values exactly halfway between two floats (ties to even), the edges of the
FP32 normal range, overflow to infinity, signed zeros, subnormal results,
infinities and NaNs (the last ones take the hardware conversion in the
kernel, the numpy cast here).  The device code itself is checked through the
kernels that use it (the mixed leaf application against the FMA kernel and
the oracle's Utilde, the streamed inputs against the plain ones)."""
import numpy as np

M32 = np.uint64(0xFFFFFFFF)


def f64_to_f32_rn(d):
    d = np.asarray(d, dtype=np.float64)
    u = d.view(np.uint64)
    hi = (u >> np.uint64(32)).astype(np.uint32)
    lo = (u & M32).astype(np.uint32)
    ahi = hi & np.uint32(0x7FFFFFFF)
    # double exponent 897 .. 1150: an FP32 normal result (or a carry to infinity)
    fast = (ahi - np.uint32(897 << 20)) < np.uint32((1151 - 897) << 20)
    # __funnelshift_l(lo, ahi, 3): the top 32 bits of (ahi:lo) << 3
    funnel = (((ahi.astype(np.uint64) << np.uint64(32)) | lo.astype(np.uint64)) >> np.uint64(29)) & M32
    bits = ((funnel - np.uint64(0xC0000000)) & M32).astype(np.uint32)
    up = (((lo & np.uint32(0x1FFFFFFF)).astype(np.uint64) + np.uint64(0x0FFFFFFF)
           + (bits & np.uint32(1)).astype(np.uint64)) >> np.uint64(29)).astype(np.uint32)
    out = ((bits + up) | (hi & np.uint32(0x80000000))).view(np.float32).copy()
    zero = (ahi == 0) & (lo == 0)
    out[zero] = hi[zero].view(np.float32)
    slow = ~fast & ~zero
    with np.errstate(over="ignore"):
        out[slow] = d[slow].astype(np.float32)
    return out, fast


def same_bits(a, b):
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))


def check(x):
    got, fast = f64_to_f32_rn(x)
    with np.errstate(over="ignore"):
        ref = np.asarray(x, dtype=np.float64).astype(np.float32)
    bad = ~same_bits(got, ref)
    assert not bad.any(), (np.asarray(x)[bad][:5], got[bad][:5], ref[bad][:5])
    return fast


def test_random_magnitudes_across_the_double_range():
    rng = np.random.default_rng(0)
    x = rng.standard_normal(400_000) * 10.0 ** rng.uniform(-60, 60, 400_000)
    fast = check(x)
    assert 0.5 < fast.mean() < 1.0  # both paths taken


def test_ties_round_to_even_and_neighbours():
    rng = np.random.default_rng(1)
    f = (rng.standard_normal(200_000) * 10.0 ** rng.uniform(-30, 30, 200_000)).astype(np.float32)
    f = f[np.isfinite(f) & (np.abs(f) > np.float32(2.0 ** -125))]
    f64 = f.astype(np.float64)
    half = np.spacing(np.abs(f)).astype(np.float64) / 2
    for x in (f64, f64 + half, f64 - half, f64 + half * (1 + 2.0 ** -20), f64 + half * (1 - 2.0 ** -20)):
        assert check(x).all()


def test_edges_of_the_fp32_range_and_special_values():
    big = float(np.finfo(np.float32).max)
    tiny = float(np.finfo(np.float32).tiny)
    x = np.array([0.0, -0.0, 1.0, -1.0, big, -big, big * (1 + 2.0 ** -25), big * (1 + 2.0 ** -24),
                  2.0 ** 128, -(2.0 ** 128), tiny, -tiny, tiny * (1 - 2.0 ** -30), tiny / 2, 2.0 ** -149,
                  2.0 ** -150, 2.0 ** -151, 1e-300, -1e-300, 1e300, np.inf, -np.inf, np.nan,
                  1 + 2.0 ** -24, 1 + 3 * 2.0 ** -24, -(1 + 3 * 2.0 ** -24), 1 + 2.0 ** -24 + 2.0 ** -52])
    check(x)
