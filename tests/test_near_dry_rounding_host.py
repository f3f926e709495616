"""The property the Float32 kernels' near-dry velocities rest on, checked on the
host: for Float32 operands, the IEEE Float64 quotient rounded to Float32 equals
the correctly rounded Float32 quotient (double rounding of a quotient from 53
to 24 bits is innocuous because 53 >= 2*24). numpy's float32 division is the
IEEE correctly rounded one, so the two sides are computed independently of
the library. The device-side check of the kernels' own function is
tests/test_gpu_near_dry_quotients.py.
"""
import numpy as np

F32_MIN_NORMAL = np.float32(1.1754944e-38)


def normal(a, b):
    with np.errstate(all="ignore"):
        q = a.astype(np.float64) / b.astype(np.float64)
    ok = (np.isfinite(a) & np.isfinite(b) & (np.abs(a) >= F32_MIN_NORMAL) & (np.abs(b) >= F32_MIN_NORMAL)
          & (np.abs(q) >= 2.0 * F32_MIN_NORMAL) & (np.abs(q) < 3.0e38))
    return a[ok], b[ok]


def check(a, b):
    a, b = normal(a, b)
    with np.errstate(all="ignore"):
        once = a / b
        twice = (a.astype(np.float64) / b.astype(np.float64)).astype(np.float32)
    assert once.dtype == np.float32
    bad = once.view(np.uint32) != twice.view(np.uint32)
    assert not bad.any(), (int(bad.sum()), a[bad][:4], b[bad][:4])
    return a.size


def test_random_bit_patterns():
    rng = np.random.default_rng(21)
    n = 2_000_000
    a = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    b = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    assert check(a, b) > n // 4


def test_quotients_closest_to_rounding_midpoints():
    """Of 4 M pairs, the 200 k whose exact quotient lies closest to a Float32
    rounding midpoint (m*b is exact in Float64 for a 25-bit midpoint m)."""
    rng = np.random.default_rng(22)
    n = 4_000_000
    b = (rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-20, 20, n))).astype(np.float32)
    m = (rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-20, 20, n))).astype(np.float32)
    mid = m.astype(np.float64) + np.spacing(m).astype(np.float64) * 0.5
    prod = mid * b.astype(np.float64)
    a = prod.astype(np.float32)
    closeness = np.abs(a.astype(np.float64) - prod) / np.spacing(a).astype(np.float64)
    keep = np.argsort(closeness)[:200_000]
    assert check(a[keep], b[keep]) > 190_000


def test_near_dry_magnitudes():
    rng = np.random.default_rng(23)
    n = 1_000_000
    hs = np.concatenate([rng.uniform(5e-6, 2e-5, n // 2), rng.uniform(5e-4, 2e-3, n - n // 2)]).astype(np.float32)
    hu = (rng.standard_normal(n) * np.exp(rng.uniform(np.log(1e-12), np.log(1e-2), n))).astype(np.float32)
    assert check(hu, hs) > n - n // 100
