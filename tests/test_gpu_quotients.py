"""The Float64 quotient of every Float64 kernel (correctly rounded reciprocals
shared by a divisor's quotients; the IEEE division for the operands that
method excludes) against IEEE division, bit for bit, on the inputs that could
break it: random bit patterns over the whole exponent range, divisors whose
significand is all ones or nearly so, numerators and divisors at the edges of
the +-500 exponent window, zeros of both signs, subnormals, infinities, NaNs,
and the magnitudes the shallow-water step divides (depths down to kappa/2,
wave-speed spreads, 1 - dt*S)."""
import ctypes as C

import numpy as np
import pytest

from volumefluxes_sm103 import _native as N

pytestmark = pytest.mark.gpu


def quotients(a, b):
    lib = N.load()
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    q = np.empty_like(a)
    rc = lib.vf_selftest_quotients(0, N.ptr(a), N.ptr(b), a.size, N.ptr(q))
    assert rc == N.VF_OK, lib.vf_last_error(None)
    return q


def same_bits(q, want):
    qb, wb = q.view(np.uint64), want.view(np.uint64)
    return (qb == wb) | (np.isnan(q) & np.isnan(want))


def from_bits(u):
    return np.asarray(u, dtype=np.uint64).view(np.float64)


def check(a, b):
    with np.errstate(all="ignore"):
        want = a / b
    q = quotients(a, b)
    bad = ~same_bits(q, want)
    assert not bad.any(), (int(bad.sum()), a[bad][:4], b[bad][:4], q[bad][:4], want[bad][:4])


def test_random_bit_patterns():
    rng = np.random.default_rng(1)
    n = 4_000_000
    check(from_bits(rng.integers(0, 2**64, n, dtype=np.uint64)), from_bits(rng.integers(0, 2**64, n, dtype=np.uint64)))


def test_moderate_exponents():
    """Both operands inside the window where the reciprocal method applies."""
    rng = np.random.default_rng(2)
    n = 4_000_000
    a = rng.standard_normal(n) * np.exp2(rng.integers(-300, 300, n))
    b = rng.standard_normal(n) * np.exp2(rng.integers(-300, 300, n))
    check(a, b)


def test_significands_near_all_ones_and_powers_of_two():
    rng = np.random.default_rng(3)
    n = 1_000_000
    e = rng.integers(1023 - 520, 1023 + 520, n).astype(np.uint64) << np.uint64(52)
    low = np.uint64((1 << 52) - 1)
    tails = np.concatenate([low - rng.integers(0, 64, n // 2).astype(np.uint64),
                            rng.integers(0, 64, n - n // 2).astype(np.uint64)])
    sign = (rng.integers(0, 2, n).astype(np.uint64) << np.uint64(63))
    b = from_bits(sign | e | tails)
    a = rng.standard_normal(n) * np.exp2(rng.integers(-40, 40, n))
    check(a, b)
    check(b, a)


def test_exponent_window_edges_and_special_values():
    rng = np.random.default_rng(4)
    edge = np.concatenate([np.exp2(np.arange(-530.0, -470.0)), np.exp2(np.arange(470.0, 530.0))])
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                         1.7976931348623157e308, 1.0, -1.0, 0.5, 2.0])
    vals = np.concatenate([edge, -edge, specials, rng.standard_normal(200)])
    a, b = np.meshgrid(vals, vals)
    check(a.ravel(), b.ravel())


def test_magnitudes_of_the_step():
    """Depths between kappa/2 and 10 m, momenta, wave-speed spreads from kappa
    to 100 m/s, and 1 - dt*S from 1 to 1e10, as the step divides them."""
    rng = np.random.default_rng(5)
    n = 2_000_000
    num = rng.standard_normal(n) * np.exp(rng.uniform(np.log(1e-12), np.log(1e2), n))
    den = np.concatenate([np.exp(rng.uniform(np.log(5e-6), np.log(10.0), n // 2)),
                          np.exp(rng.uniform(np.log(1e-5), np.log(1e10), n - n // 2))])
    check(num, den)
    check(np.zeros(n) * np.sign(num), den)
