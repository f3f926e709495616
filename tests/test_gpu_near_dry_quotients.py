"""The near-dry velocity quotient of the Float32 kernels against the IEEE
Float64 division rounded to Float32, bit for bit, both computed on the device.

Face sides and cells of a Float32 state with |h| below the near-dry threshold
divide (hu, hv) by the desingularised depth h* with the Float64 quotient's
bits (src/equations/equation.jl:40-67 is the division; the Float64 step is
asked for because a thin film's velocity is a quotient of two small numbers).
The kernels get those bits from the correctly rounded Float32 quotient, which
equals the Float64 quotient rounded to Float32 because double rounding of a
quotient from 53 to 24 bits is innocuous (53 >= 2*24). These cases check the
claim where it could fail: random Float32 bit patterns with normal operands
and quotients, quotients close to Float32 rounding midpoints, and the
magnitudes a near-dry face divides.
"""
import numpy as np
import pytest

from volumefluxes_sm103 import _native as N

pytestmark = pytest.mark.gpu

F32_MIN_NORMAL = np.float32(1.1754944e-38)


def quotients(a, b):
    lib = N.load()
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    q = np.empty_like(a)
    q64 = np.empty_like(a)
    rc = lib.vf_selftest_near_dry_quotients(0, N.ptr(a), N.ptr(b), a.size, N.ptr(q), N.ptr(q64))
    assert rc == N.VF_OK, lib.vf_last_error(None)
    return q, q64


def normal_cases(a, b):
    """Keep pairs whose operands and Float64 quotient are finite normal Float32
    numbers (the Float32 kernels flush subnormals to zero)."""
    a = np.asarray(a, dtype=np.float32)
    b = np.asarray(b, dtype=np.float32)
    with np.errstate(all="ignore"):
        exact = a.astype(np.float64) / b.astype(np.float64)
    ok = (np.isfinite(a) & np.isfinite(b) & (np.abs(a) >= F32_MIN_NORMAL) & (np.abs(b) >= F32_MIN_NORMAL)
          & (np.abs(exact) >= 2.0 * F32_MIN_NORMAL) & (np.abs(exact) < 3.0e38))
    return a[ok], b[ok], exact[ok]


def check(a, b, min_cases):
    a, b, exact = normal_cases(a, b)
    assert a.size >= min_cases
    q, q64 = quotients(a, b)
    bad = q.view(np.uint32) != q64.view(np.uint32)
    assert not bad.any(), (int(bad.sum()), a[bad][:4], b[bad][:4], q[bad][:4], q64[bad][:4])
    # and both are the host's IEEE Float64 quotient rounded to Float32
    want = exact.astype(np.float32)
    host_bad = q.view(np.uint32) != want.view(np.uint32)
    assert not host_bad.any(), (int(host_bad.sum()), a[host_bad][:4], b[host_bad][:4])


def test_random_bit_patterns():
    rng = np.random.default_rng(11)
    n = 4_000_000
    a = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    b = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    check(a, b, n // 4)


def test_quotients_near_rounding_midpoints():
    """Pairs whose exact quotient lies closest to a Float32 rounding midpoint:
    for a midpoint m (25 significant bits) and a divisor b (24), m*b is exact
    in Float64, and a = RN32(m*b) leaves a/b - m = (a - m*b)/b; of 8 M random
    pairs keep the 400 k with the smallest |a - m*b| relative to ulp(a)."""
    rng = np.random.default_rng(12)
    n = 8_000_000
    b = (rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-20, 20, n))).astype(np.float32)
    m = (rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-20, 20, n))).astype(np.float32)
    mid = m.astype(np.float64) + np.spacing(m).astype(np.float64) * 0.5
    prod = mid * b.astype(np.float64)
    a = prod.astype(np.float32)
    closeness = np.abs(a.astype(np.float64) - prod) / np.spacing(a).astype(np.float64)
    keep = np.argsort(closeness)[:400_000]
    check(a[keep], b[keep], 390_000)


def test_magnitudes_of_near_dry_faces():
    """Desingularised depths from kappa/2 to 2*kappa-ish (kappa = 1e-5 and
    1e-3) and momenta of thin films and of faster flow."""
    rng = np.random.default_rng(13)
    n = 2_000_000
    hs = np.concatenate([rng.uniform(5e-6, 2e-5, n // 2), rng.uniform(5e-4, 2e-3, n - n // 2)]).astype(np.float32)
    hu = (rng.standard_normal(n) * np.exp(rng.uniform(np.log(1e-12), np.log(1e-2), n))).astype(np.float32)
    check(hu, hs, n - n // 100)
