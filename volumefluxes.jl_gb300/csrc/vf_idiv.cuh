// vf_idiv.cuh -- IEEE double division on the integer pipe.
//
// GB300 issues Float64 at 2 operations per clock per SM, and a correctly
// rounded Float64 division costs about ten of them; the integer and Float32
// pipes sit idle in the Float64 step kernels. This computes q = RN(a / b) for
// normal operands with integer arithmetic:
//   1. significands ma, mb in [2^52, 2^53); ma doubled when ma < mb, so ma/mb in [1, 2);
//   2. y ~ 2^127 / (mb << 11): a 24-bit Float32 reciprocal seed refined by two
//      fixed-point Newton steps (y += y*(1 - d*y)), accurate to ~2^-60;
//   3. q ~ floor(ma * 2^52 / mb) = mulhi(ma, y), then the exact remainder
//      r = ma*2^52 - q*mb (it fits 64 bits) corrects q by up to two units;
//   4. round to nearest even from 2r vs mb, carry into the exponent.
// Steps 3-4 make the result the correctly rounded quotient whatever the
// seed's last bits, so host and device agree although their Float32 seeds may
// differ. Zero numerators return signed zeros; every other non-normal operand
// or result (subnormal, zero divisor, infinity, NaN, overflow, underflow) takes
// the hardware division. The same source compiles for the host, where the
// tests compare it bit for bit with IEEE division.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define VF_HD __host__ __device__ __forceinline__
#else
#define VF_HD inline
#endif

namespace vf {

VF_HD uint64_t idiv_mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

VF_HD uint64_t idiv_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}

VF_HD double idiv_double(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

// Reciprocal seed of xf in [0.5, 1): about 22 correct bits are enough.
VF_HD float idiv_rcp_seed(float xf) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(xf));
  return r;
#elif defined(VF_IDIV_SEED_SCALE)
  return (1.0f / xf) * (float)(VF_IDIV_SEED_SCALE);  // host tests: a deliberately perturbed seed
#else
  return 1.0f / xf;
#endif
}

// Correctly rounded a / b, or false when the operands or the result leave the
// normal range (the caller then divides in hardware).
VF_HD bool idiv_normal(double a, double b, double* out) {
  const uint64_t FRAC = (1ull << 52) - 1, HID = 1ull << 52;
  const uint64_t ua = idiv_bits(a), ub = idiv_bits(b);
  const uint64_t sign = (ua ^ ub) & 0x8000000000000000ull;
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
  if (eb - 1u >= 0x7feu) return false;               // b zero, subnormal, inf or nan
  if (ea - 1u >= 0x7feu) {
    if (ea == 0 && (ua & FRAC) == 0) {               // +-0 / normal = signed zero
      *out = idiv_double(sign);
      return true;
    }
    return false;
  }
  uint64_t ma = (ua & FRAC) | HID;
  const uint64_t mb = (ub & FRAC) | HID;
  int e = (int)ea - (int)eb + 1023;
  if (ma < mb) {
    ma <<= 1;
    e -= 1;
  }
  // Seed: xf = (d >> 40) / 2^24 in [0.5, 1) built from bits, y0 = 2^63 + frac(1/xf) << 40.
  const uint64_t d = mb << 11;
  const uint32_t xb = 0x3f000000u | (uint32_t)((d >> 40) & 0x7fffffu);
  float xf;
#if defined(__CUDA_ARCH__)
  xf = __uint_as_float(xb);
#else
  std::memcpy(&xf, &xb, 4);
#endif
  float yf = idiv_rcp_seed(xf);                       // in (1, 2]
  uint32_t yb;
#if defined(__CUDA_ARCH__)
  yb = __float_as_uint(yf);
#else
  std::memcpy(&yb, &yf, 4);
#endif
  uint64_t y;
  if (yb >= 0x40000000u) {
    y = 0xffffffffffffffffull;                        // 1/xf == 2 (xf == 0.5): saturate
  } else if (yb < 0x3f800000u) {
    y = 1ull << 63;                                   // an approximate 1/xf just below 1
  } else {
    y = (1ull << 63) | ((uint64_t)(yb & 0x7fffffu) << 40);
  }
  // Two Newton steps on Y = y / 2^63 ~ 1 / D, D = d / 2^64: Y += Y * (1 - D * Y).
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const uint64_t p = idiv_mulhi(d, y);              // D*Y * 2^63
    if (p <= (1ull << 63)) {
      const uint64_t eps = (1ull << 63) - p;
      const uint64_t inc = idiv_mulhi(y, eps) << 1;
      y = (y + inc < y) ? 0xffffffffffffffffull : y + inc;
    } else {
      const uint64_t eps = p - (1ull << 63);
      y -= idiv_mulhi(y, eps) << 1;
    }
  }
  // q ~ ma * 2^63 / d = ma * y / 2^64, then the exact remainder.
  uint64_t q = idiv_mulhi(ma, y);
  int64_t r = (int64_t)((ma << 52) - q * mb);
  if (r < 0) { --q; r += (int64_t)mb; }
  if (r < 0) { --q; r += (int64_t)mb; }
  if (r >= (int64_t)mb) { ++q; r -= (int64_t)mb; }
  if (r >= (int64_t)mb) { ++q; r -= (int64_t)mb; }
  const uint64_t r2 = (uint64_t)r << 1;
  if (r2 > mb || (r2 == mb && (q & 1))) ++q;
  if (q == (HID << 1)) {
    q = HID;
    e += 1;
  }
  if (e <= 0 || e >= 0x7ff) return false;            // subnormal, underflow or overflow
  *out = idiv_double(sign | ((uint64_t)e << 52) | (q & FRAC));
  return true;
}

}  // namespace vf
