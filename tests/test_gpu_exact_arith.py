"""The stage kernels' FP64 division and square root against IEEE arithmetic.

The per-pair work of the stages needs a correctly rounded FP64 division and square root
for every pair in range.  On GB300 the FP64 pipe issues a small fraction of the FP32
rate, so the kernels compute both on the FP32 and integer pipes (a float-float estimate
corrected by the exact integer remainder of the significands).  They must return the
IEEE result bit for bit: the host's division and square root (numpy) are the check, on
random operands over a wide exponent range, on the operand shapes of the stages, and on
the special values that take the FP64 fallback.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _random_doubles(rng, n, emin, emax, signed=False):
    mant = rng.integers(0, 1 << 52, size=n, dtype=np.uint64)
    exp = rng.integers(emin + 1023, emax + 1023, size=n).astype(np.uint64)
    bits = (exp << np.uint64(52)) | mant
    if signed:
        bits |= rng.integers(0, 2, size=n).astype(np.uint64) << np.uint64(63)
    return bits.view(np.float64)


def _check(a, b):
    from openmps_gb300.computer import exact_arith

    q, r = exact_arith(a, b)
    with np.errstate(all="ignore"):
        qr = a / b
        rr = np.sqrt(a)
    bad_q = q.view(np.uint64) != qr.view(np.uint64)
    bad_r = r.view(np.uint64) != rr.view(np.uint64)
    # NaN payloads may differ: any NaN matches any NaN
    bad_q &= ~(np.isnan(q) & np.isnan(qr))
    bad_r &= ~(np.isnan(r) & np.isnan(rr))
    assert not bad_q.any(), "division differs for %s / %s" % (a[bad_q][:3], b[bad_q][:3])
    assert not bad_r.any(), "square root differs for %s" % a[bad_r][:3]


def test_random_operands(gpu_lib):
    rng = np.random.default_rng(20261204)
    n = 4_000_000
    a = _random_doubles(rng, n, -500, 500, signed=True)
    b = _random_doubles(rng, n, -500, 500, signed=True)
    _check(a, b)
    # significands close to each other, all ones, powers of two
    near = (a.view(np.uint64) ^ rng.integers(0, 1 << 12, size=n, dtype=np.uint64)).view(np.float64)
    _check(a, near)
    ones = (a.view(np.uint64) | np.uint64((1 << 52) - 1)).view(np.float64)
    pow2 = (b.view(np.uint64) & ~np.uint64((1 << 52) - 1)).view(np.float64)
    _check(ones, pow2)
    _check(pow2, ones)
    # squares and their neighbours (roots close to a rounding boundary)
    root = _random_doubles(rng, n, -200, 200)
    sq = root * root
    for k in (-2, -1, 0, 1, 2):
        _check((sq.view(np.int64) + k).view(np.float64), root)


def test_stage_operands(gpu_lib):
    # r2 = dx^2 + dz^2 of pairs within a few l0 of each other, r = sqrt(r2), re / r and
    # c / (r r r), as the density, source, viscosity and PPE coefficients form them
    from openmps_gb300.computer import exact_arith

    rng = np.random.default_rng(7)
    n = 2_000_000
    for l0 in (5e-4, 2.5e-3, 1e-2):
        dx = rng.uniform(-4.8 * l0, 4.8 * l0, n)
        dz = rng.uniform(-4.8 * l0, 4.8 * l0, n)
        r2 = dx * dx + dz * dz
        _, r = exact_arith(r2, np.ones(n))
        assert np.array_equal(r.view(np.uint64), np.sqrt(r2).view(np.uint64))
        _check(np.full(n, 4.0 * l0), r)
        _check(np.full(n, 3.0 * 1e-6 * 4.0 * l0 / 35.609223), (r * r) * r)
        _check(dx * rng.normal(size=n), (r * r) * r)


def test_special_values(gpu_lib):
    tiny = np.finfo(np.float64).tiny
    vals = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, tiny, tiny / 3, 5e-324, np.finfo(np.float64).max,
                     1e308, 1e-308, 2.0 ** -1022, 2.0 ** 1023, 3.0, 0.1], dtype=np.float64)
    a = np.repeat(vals, vals.size)
    b = np.tile(vals, vals.size)
    _check(a, b)
