"""The bit-level double -> (hi, lo) float split of csrc/kernels.cuh
(df_split), restated with numpy integer arithmetic and checked against
numpy's round-to-nearest-even conversions on 2 M doubles over the exponent
fields the fast path covers (949 .. 1149), with forced ties and carries.

The split must equal hi = fl32(v), lo = fl32(v - hi) bit for bit: the
53-bit significand splits into its top 24 bits K and low 29 bits R, K
rounds to nearest even on R (a carry out of K moves into the float exponent
field), and v - hi is the remainder r = R or R - 2^29 in units of
2^(e - 1075), which one int -> float conversion rounds and a power of two
scales exactly.  tests/test_gpu_split.py checks the CUDA function itself on
the device."""
import numpy as np


def split_bits(u):
    e = ((u >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    m = (u & np.uint64(0xFFFFFFFFFFFFF)) | np.uint64(0x10000000000000)
    k = (m >> np.uint64(29)).astype(np.int64)
    rr = (m & np.uint64(0x1FFFFFFF)).astype(np.int64)
    up = (rr > 0x10000000) | ((rr == 0x10000000) & ((k & 1) == 1))
    k = np.where(up, k + 1, k)
    r = np.where(up, rr - 0x20000000, rr)
    neg = (u >> np.uint64(63)).astype(np.int64)
    bits = (neg << 31) | (((e - 896) << 23) + (k - 0x800000))
    hi = (bits & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    scale = ((e - 948) << 23).astype(np.uint32).view(np.float32)
    lo = np.where(neg == 1, -r, r).astype(np.float32) * scale
    return hi, lo


def test_split_matches_round_to_nearest_even():
    rng = np.random.default_rng(7)
    n = 2_000_000
    mant = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    exps = rng.integers(949, 1150, n, dtype=np.uint64)
    sign = rng.integers(0, 2, n, dtype=np.uint64)
    u = (sign << np.uint64(63)) | (exps << np.uint64(52)) | mant
    t = n // 8
    u[:t] = (u[:t] & ~np.uint64(0x1FFFFFFF)) | np.uint64(0x10000000)     # ties in the rounded bits
    u[t:2 * t] = u[t:2 * t] | np.uint64(0xFFFFFFFFFFFFF)                # carries into the exponent
    u[2 * t:3 * t] = u[2 * t:3 * t] & ~np.uint64(0x1FFFFFFF)            # exact halves: lo = 0
    v = u.view(np.float64)
    ref_hi = v.astype(np.float32)
    ref_lo = (v - ref_hi.astype(np.float64)).astype(np.float32)
    hi, lo = split_bits(u)
    np.testing.assert_array_equal(hi.view(np.uint32), ref_hi.view(np.uint32))
    np.testing.assert_array_equal(lo.view(np.uint32), ref_lo.view(np.uint32))
