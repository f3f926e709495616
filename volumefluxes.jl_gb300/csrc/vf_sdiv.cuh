// vf_sdiv.cuh -- correctly rounded Float64 quotients that share a divisor.
//
// The flux and friction arithmetic divides several numerators by one value
// (u = hu/h*, v = hv/h*; the four central-upwind terms over a+ - a-; the two
// momenta over 1 - dt*S). This computes the divisor's reciprocal once and
// each quotient in four FP64-pipe operations, with the result still the
// correctly rounded a/b (a build option, VF_FP64_SHARED_DIV; the step kernels
// measured faster with one IEEE division per quotient):
//   1. y ~ 1/b: a hardware reciprocal seed (rcp.approx.ftz.f64) refined by two
//      Newton-Raphson steps e = 1 - b*y, y += e*y (each an FMA pair);
//   2. q0 = a*y, r = a - b*q0 (FMA, exact when q0 is within an ulp), and
//      q = q0 + r*y: the correction step of Markstein's division method
//      (P. Markstein, IBM J. Res. Dev. 34(1), 1990; Muller et al., Handbook of
//      Floating-Point Arithmetic, ch. 5);
//   3. an exact rounding test decides whether q is RN(a/b): with r2 = a - b*q
//      (exact when q is within an ulp), q is the correctly rounded quotient
//      iff |r2| < ulp(q)/2 * |b|, or |r2| == ulp(q)/2 * |b| and q is even
//      (ties to even). ulp(q)/2 * |b| is |b| scaled by a power of two, so the
//      test itself is exact;
//   4. when the test fails, q is normally the neighbour of RN(a/b): with y
//      within a few ulps of 1/b, |q - a/b| < ulp(q) and the true quotient lies
//      between q and its neighbour on the side of r2/b, so RN(a/b) is that
//      neighbour (for a tie the even one, again the neighbour since q is odd
//      there), one step of q's bit pattern away; the same exact test confirms
//      it before it is used.
// When an operand or the result is outside the range where the scaled bound is
// exact (zero divisor, subnormals, huge or tiny exponents, q a power of two,
// where the ulp below q is half the one above), the hardware division is used
// instead, so the result always equals IEEE a/b. Zero numerators give the
// signed zero directly. The same source compiles for the host, where tests
// compare it with IEEE division bit for bit.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define VF_SD __host__ __device__ __forceinline__
#else
#define VF_SD inline
#endif

namespace vf {

VF_SD uint64_t sd_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}

VF_SD double sd_double(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

VF_SD double sd_fma(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
  return __fma_rn(a, b, c);
#else
  return __builtin_fma(a, b, c);
#endif
}

// Seed reciprocal, a few correct bits are enough.
VF_SD double sd_seed(double b) {
#if defined(__CUDA_ARCH__)
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(b));
  return r;
#elif defined(VF_SDIV_SEED_SCALE)
  return (double)(float)(1.0 / b) * (double)(VF_SDIV_SEED_SCALE);  // host tests: a deliberately poor seed
#else
  return (double)(float)(1.0 / b);
#endif
}

struct SharedRecip {
  double b, y;
  int eb;  // biased exponent of b; 0 marks "divide in hardware"
};

VF_SD SharedRecip sd_recip(double b) {
  SharedRecip R;
  R.b = b;
  R.y = 0.0;
  const int eb = (int)((sd_bits(b) >> 52) & 0x7ff);
  // b normal with a moderate exponent: y and the scaled bound stay normal.
  R.eb = (eb > 64 && eb < 2000) ? eb : 0;
  if (R.eb) {
    double y = sd_seed(b);
    double e = sd_fma(-b, y, 1.0);
    y = sd_fma(e, y, y);
    e = sd_fma(-b, y, 1.0);
    R.y = sd_fma(e, y, y);
  }
  return R;
}

// Whether q is RN(a/b), by the exact test of step 3; false also when q or the
// scaled bound leaves the range where the test is exact (*in_range = false).
VF_SD bool sd_is_rn(const SharedRecip& R, double a, double q, double* r2_out, bool* in_range) {
  const uint64_t uq = sd_bits(q);
  const int eq = (int)((uq >> 52) & 0x7ff);
  const uint64_t fq = uq & ((1ull << 52) - 1);
  // ulp(q)/2 * |b| = |b| * 2^(eq - 1023 - 53): keep it normal and q off a binade edge.
  const int es = R.eb + eq - 1023 - 53;
  *in_range = !(fq == 0 || eq < 64 || eq > 2000 || es < 2 || es > 2045);
  if (!*in_range) return false;
  const double hb = sd_double((uint64_t)es << 52 | (sd_bits(R.b) & ((1ull << 52) - 1)));
  const double r2 = sd_fma(-R.b, q, a);
  *r2_out = r2;
  const uint64_t ar2 = sd_bits(r2) & 0x7fffffffffffffffull, ahb = sd_bits(hb);
  return ar2 < ahb || (ar2 == ahb && (fq & 1) == 0);
}

// The correctly rounded a / b when the fast path can prove it (true), else false.
VF_SD bool sd_div_fast(const SharedRecip& R, double a, double* out) {
  const uint64_t ua = sd_bits(a);
  if ((ua << 1) == 0) {  // +-0 / b: the signed zero
    *out = sd_double((ua ^ sd_bits(R.b)) & 0x8000000000000000ull);
    return true;
  }
  if (R.eb == 0) return false;
  const double q0 = a * R.y;
  const double r = sd_fma(-R.b, q0, a);
  const double q = sd_fma(r, R.y, q0);
  double r2 = 0.0;
  bool in_range;
  if (sd_is_rn(R, a, q, &r2, &in_range)) {
    *out = q;
    return true;
  }
  if (!in_range) return false;
  // Step 4: the neighbour on the side of the true quotient (|a/b| > |q| iff
  // r2/b has q's sign), checked by the same exact test.
  const uint64_t uq = sd_bits(q);
  const bool up = ((sd_bits(r2) ^ sd_bits(R.b) ^ uq) >> 63) == 0;
  const double qn = sd_double(up ? uq + 1 : uq - 1);
  double r3;
  if (sd_is_rn(R, a, qn, &r3, &in_range)) {
    *out = qn;
    return true;
  }
  return false;
}

// IEEE a / b for a divisor prepared with sd_recip.
VF_SD double sd_div(const SharedRecip& R, double a) {
  double q;
  return sd_div_fast(R, a, &q) ? q : a / R.b;
}

}  // namespace vf
