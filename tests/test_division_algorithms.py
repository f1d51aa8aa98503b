"""The device arithmetic helpers' algorithms, restated on the CPU with exact
arithmetic (no GPU needed): each test replays the steps the device code
takes, with a fused multiply-add rounded once from the exact value, and
checks the property the device code relies on.  The device implementations
themselves are checked against CUDA's and numpy's results in
test_division_gpu.py and test_multidim_gpu.py.
"""

from fractions import Fraction

import numpy as np


def _fma(a, b, c):
    """a * b + c rounded once to the nearest double (Python's int / int
    division rounds correctly, and so does float(Fraction))."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _ulps(a, b):
    return abs(int(np.float64(a).view(np.int64)) -
               int(np.float64(b).view(np.int64)))


def _operands(rng, n, lo, hi):
    bits = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    e = rng.integers(1023 + lo, 1023 + hi, n, dtype=np.uint64)
    s = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    return (bits | (e << np.uint64(52)) | s).view(np.float64)


def test_markstein_quotient_from_tabulated_reciprocal_is_exact():
    """div_rcp: q0 = x r, then two corrections q + (x - q d) r by FMA, from
    r = 1 / d rounded to nearest, gives exactly the IEEE quotient (random
    operands, quotients next to a rounding midpoint, divisors of all-ones
    significand)."""
    rng = np.random.default_rng(2)
    x = _operands(rng, 1500, -60, 60)
    d = _operands(rng, 1500, -60, 60)
    mid = _operands(rng, 500, -20, 20)
    mid = mid + np.spacing(mid) / 2          # halfway between two doubles
    dm = _operands(rng, 500, -20, 20)
    x = np.concatenate([x, mid * dm, np.full(100, 1.0), rng.uniform(1, 2, 100)])
    d = np.concatenate([d, dm, np.nextafter(2.0, 0) * rng.choice([1, -0.5, 4], 100),
                        np.nextafter(2.0, 0) * np.ones(100)])
    for xv, dv in zip(x.tolist(), d.tolist()):
        r = 1.0 / dv
        q = xv * r
        q = _fma(_fma(-q, dv, xv), r, q)
        q = _fma(_fma(-q, dv, xv), r, q)
        assert q == xv / dv, (xv, dv)


def test_newton_reciprocal_from_a_coarse_seed_is_within_one_ulp():
    """recip: two Newton steps r + r (1 - d r) by FMA from an FP32 estimate
    of 1 / (d's significand) put r within one ulp of 1 / d.  The hardware
    estimate is within about 2^-22; the seeds here are the correctly rounded
    FP32 reciprocal moved by up to 8 FP32 ulps (~2^-20), coarser still."""
    rng = np.random.default_rng(3)
    d = _operands(rng, 2000, -1000, 1000)
    worst = 0
    for dv in d.tolist():
        m, e = np.frexp(abs(dv))              # |d| = m 2^e, m in [0.5, 1)
        sig = np.float32(2 * m)               # top 24 bits of the significand
        seed = np.float32(1) / sig
        seed = np.nextafter(seed, np.float32(np.inf if rng.integers(2) else 0),
                            dtype=np.float32)
        for _ in range(int(rng.integers(0, 8))):
            seed = np.nextafter(seed, np.float32(2), dtype=np.float32)
        r = float(np.ldexp(np.float64(seed), 1 - int(e)))
        r = -r if dv < 0 else r
        t = _fma(-dv, r, 1.0)
        r = _fma(r, t, r)
        t = _fma(-dv, r, 1.0)
        r = _fma(r, t, r)
        worst = max(worst, _ulps(r, 1.0 / dv))
    assert worst <= 1


def test_geometry_rounding_without_range_select_is_round_to_nearest_even():
    """geo_r: adding 2^28 - 1 plus the lowest kept bit to the 64-bit pattern,
    taking bits 29..60 and rebiasing the exponent modulo 2^32 is IEEE
    round-to-nearest-even for every double in FP32's normal range (ties,
    near-ties and carries into the exponent included); below the range the
    compare-and-select gives a signed zero."""
    rng = np.random.default_rng(4)
    n = 400000
    bits = rng.integers(0, 1 << 63, n, dtype=np.uint64)
    exp = rng.integers(880, 1151, n, dtype=np.uint64)
    bits = (bits & ~np.uint64(0x7FF << 52)) | (exp << np.uint64(52))
    low = np.uint64(0x1FFFFFFF)
    for k, pat in enumerate((0x10000000, 0x0FFFFFFF, 0x10000001)):
        sl = slice(k * 40000, (k + 1) * 40000)
        bits[sl] = (bits[sl] & ~low) | np.uint64(pat)
    bits[120000:160000] |= np.uint64((1 << 52) - 1)
    x = bits.view(np.float64)
    hi = (bits >> np.uint64(32)).astype(np.uint32)
    t = bits + np.uint64(0x0FFFFFFF) + ((bits >> np.uint64(29)) & np.uint64(1))
    r = ((t >> np.uint64(29)) & np.uint64(0xFFFFFFFF)).astype(np.uint32) \
        - np.uint32(0xC0000000)
    keep = (hi & np.uint32(0x7FF00000)) >= np.uint32(897 << 20)
    r = np.where(keep, r, np.uint32(0)) | (hi & np.uint32(0x80000000))
    got = r.view(np.float32)
    with np.errstate(over="ignore"):
        want = x.astype(np.float32)
    normal = (exp >= 897) & (exp <= 1150)
    assert (got[normal].view(np.uint32) == want[normal].view(np.uint32)).all()
    tiny = exp < 897
    assert (got[tiny] == 0).all()
    assert (np.signbit(got[tiny]) == np.signbit(x[tiny])).all()
