"""CPU check of the panel-subdivision threshold rule used by the coefficient kernels
(o3g_coeff.cu, farther_rn): `sqrt_rn(d2) > thr` is decided from d2 against thr * thr
whenever the two differ by more than 2^-20 relative, and by the correctly rounded square
root only inside that band.  numpy's float32 products and square roots round like the
device's __fmul_rn and __fsqrt_rn, so the rule is emulated here on d2 values packed
around the boundary, over thresholds across many binades, including powers of two and
their predecessors (where the float spacing changes)."""
import numpy as np


def _farther(d2, thr):
    f = np.float32
    thr2 = (thr * thr).astype(f)
    hi = (thr2 * f(1.00000095367431640625)).astype(f)
    lo = (thr2 * f(0.99999904632568359375)).astype(f)
    exact = np.sqrt(d2) > thr
    return np.where(d2 > hi, True, np.where(d2 < lo, False, exact)), exact


def test_squared_threshold_rule_matches_rounded_sqrt():
    rng = np.random.default_rng(11)
    f = np.float32
    for e in range(-24, 24, 3):
        base = f(2.0 ** e)
        thr = np.concatenate([base * (1 + rng.random(100000).astype(f)),
                              np.full(500, np.nextafter(base, f(0))), np.full(500, base)]).astype(f)
        thr2 = (thr.astype(np.float64) ** 2)
        for width in (2.0 ** -17, 2.0 ** -21, 2.0 ** -24):
            rel = (rng.random(thr.size) * 2 - 1) * width
            d2 = (thr2 * (1 + rel)).astype(f)
            fast, exact = _farther(d2, thr)
            assert np.array_equal(fast, exact), (e, width)
        # d2 exactly at the boundary of the band and at zero
        t2 = (thr * thr).astype(f)
        for d2 in (t2, (t2 * f(1.00000095367431640625)).astype(f), (t2 * f(0.99999904632568359375)).astype(f),
                   np.nextafter(t2, f(np.inf)), np.nextafter(t2, f(0)), np.zeros_like(t2)):
            fast, exact = _farther(d2.astype(f), thr)
            assert np.array_equal(fast, exact), e
