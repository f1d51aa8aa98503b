"""Device division helpers against IEEE arithmetic: the spacetime march's
quotients from tabulated reciprocals (Markstein's method, exact) and the
multi-dimensional FP64 march's Newton reciprocal (within one ulp)."""

import numpy as np
import pytest


def _division_cases():
    """x and d pairs: random significands over the whole window and beyond
    it, quotients within a hair of a rounding midpoint, divisors of all-ones
    significand, signed zeros, denormals, infinities and NaN."""
    rng = np.random.default_rng(11)
    n = 1 << 20

    def rand(exp_lo, exp_hi, size):
        bits = rng.integers(0, 1 << 52, size, dtype=np.uint64)
        e = rng.integers(exp_lo, exp_hi, size, dtype=np.uint64)
        s = rng.integers(0, 2, size, dtype=np.uint64) << np.uint64(63)
        return (bits | (e << np.uint64(52)) | s).view(np.float64)

    x = rand(1023 - 420, 1023 + 420, n)
    d = rand(1023 - 420, 1023 + 420, n)
    # Quotients next to a midpoint: x = RN(m d) for m halfway between two
    # doubles.
    k = n // 4
    m = rand(1023 - 30, 1023 + 30, k)
    mid = m + np.spacing(m) / 2
    d[:k] = rand(1023 - 30, 1023 + 30, k)
    x[:k] = mid * d[:k]
    # Divisors with every significand bit set, and exact small ratios.
    d[k:k + 1000] = np.nextafter(2.0, 0) * rng.choice([-1, 1, 0.5, 4], 1000)
    x[k + 1000:k + 2000] = d[k + 1000:k + 2000] * rng.integers(
        1, 1000, 1000)
    special = np.array([0.0, -0.0, 5e-324, -2e-310, 1e-300, 1e300, np.inf,
                        -np.inf, np.nan, 1.0, 3.0, 2.0 ** -400, 2.0 ** 400])
    ns = len(special)
    x[-ns * ns:] = np.repeat(special, ns)
    d[-ns * ns:] = np.tile(special, ns)
    return x, d


@pytest.mark.gpu
def test_division_by_tabulated_reciprocal_is_exact():
    """div_rcp (Markstein's method from a tabulated reciprocal) gives the
    IEEE quotient bit for bit: against the device's own division and
    against numpy's, over random operands across and beyond its exponent
    window, near-midpoint quotients, all-ones divisors and special values."""
    from solvcon_gb300._lib import check, lib, ptr
    x, d = _division_cases()
    n = x.size
    q = np.empty(n)
    qdiv = np.empty(n)
    rcp = np.empty(n)
    check(lib.scg_divide_check(ptr(x), ptr(d), ptr(q), ptr(qdiv), ptr(rcp),
                               n))
    with np.errstate(all="ignore"):
        want = x / d
    nan = np.isnan(want)
    assert np.isnan(q[nan]).all() and np.isnan(qdiv[nan]).all()
    ok = ~nan
    assert (qdiv[ok].view(np.uint64) == want[ok].view(np.uint64)).all()
    bad = q[ok].view(np.uint64) != want[ok].view(np.uint64)
    assert not bad.any(), list(zip(x[ok][bad][:5], d[ok][bad][:5]))


@pytest.mark.gpu
def test_march_reciprocal_within_one_ulp():
    """The FP64 march's reciprocal (Newton's iteration from the FP32
    hardware seed) is within one ulp of 1 / d for |d| in [2^-1022, 2^1022)
    of either sign, and the IEEE reciprocal outside it (zeros, subnormals,
    the largest magnitudes, infinities, NaN)."""
    from solvcon_gb300._lib import check, lib, ptr
    x, d = _division_cases()
    d = np.concatenate([d, [2.0 ** -1021, -2.0 ** -1021, np.nextafter(2.0 ** 1022, 0),
                            2.0 ** 1022, 2.0 ** -1022, 1e-310, -0.0,
                            np.finfo(float).max, np.nextafter(1.0, 2.0), 1.0,
                            np.nextafter(2.0, 0.0)]])
    x = np.ones_like(d)
    n = d.size
    q, qdiv, rcp = np.empty(n), np.empty(n), np.empty(n)
    check(lib.scg_divide_check(ptr(x), ptr(d), ptr(q), ptr(qdiv), ptr(rcp),
                               n))
    with np.errstate(all="ignore"):
        want = 1.0 / d
    e = (d.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    inside = (e >= 1) & (e <= 2044)
    gap = np.abs(rcp[inside].view(np.int64) - want[inside].view(np.int64))
    assert gap.max() <= 1, d[inside][gap > 1][:5]
    out = ~inside
    nan = np.isnan(want[out])
    assert np.isnan(rcp[out][nan]).all()
    assert (rcp[out][~nan].view(np.uint64) ==
            want[out][~nan].view(np.uint64)).all()
