// vf_math.cuh -- per-cell and per-face arithmetic of VolumeFluxes.jl's
// practical 2D shallow-water path, restated for the device.
//
// Every expression keeps the reference's operation order, because the Float64
// path must reproduce the reference bit for bit: the Float64 translation unit
// is compiled with -fmad=false, so a*b+c stays two rounded operations as in
// Julia. Float32 instances may contract and use fast reciprocals (their error
// is stated against the Float64 oracle, not claimed bitwise).
//
// GB300 executes Float64 at 1/64 of the Float32 rate, so the Float64 traits
// below move every comparison, min/max and sign test onto the integer pipe by
// comparing IEEE bit patterns; only +, -, *, /, sqrt stay on the FP64 pipe.
//
// Citations are path:line within the VolumeFluxes.jl project.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>


// Float32 reciprocals and cube roots come from the special-function unit
// (rcp.approx, and cbrt(x) = 2^(log2|x| / 3) with the sign of x; a few ulps);
// Float32 results are stated against the Float64 oracle, not claimed bitwise.
// Measured on the 4096^2 wet/dry step (Float32 is instruction-issue bound):
// 0.919 ms with the special-function unit, 1.069 ms with the correctly
// rounded reciprocal and the libm cube root.
// Float64 quotients correct to about one ulp instead of correctly rounded (1),
// for the tolerance-bound Float64 kernels (vf_f64f.cu, built with multiply-add
// contraction): a reciprocal from the hardware approximation refined by one
// third-order Newton step, a quotient a/b as a * (1/b) plus one residual
// correction, and quotients that share a divisor as products with one shared
// reciprocal. Cube roots come from the CUDA math library. 0: every operation
// rounds as in the reference (the bitwise kernels).
#ifndef VF_FP64_FAITHFUL
#define VF_FP64_FAITHFUL 0
#endif
// Correctly rounded Float64 quotients from one correctly rounded reciprocal per
// divisor (1) instead of one hardware IEEE division per quotient (0): the same
// bits, fewer FP64 instructions where several quotients share a divisor. The
// Float64 unit builds with 1: bit for bit the IEEE results on every parity
// case and over the 4096^2 wet/dry workload's 1000 steps, and 28.8 instead of
// 31.0 ms per step there (1.43x on the fully wet 256^2 dam break).
#ifndef VF_FP64_MARKSTEIN
#define VF_FP64_MARKSTEIN 0
#endif

namespace vf {

// ---------------------------------------------------------------------------
// Precision traits.
template <typename T>
struct Arith;

// Float64: exact IEEE semantics. Comparisons are done on bit patterns (valid
// for every non-NaN operand; a valid step never produces NaN because every
// divisor is bounded away from zero).
template <>
struct Arith<double> {
  static constexpr bool exact = !VF_FP64_FAITHFUL;
  static __device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }
  // Monotone key: orders all non-NaN doubles, with -0.0 just below +0.0.
  static __device__ __forceinline__ long long key(double x) {
    const long long b = bits(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
  }
  static __device__ __forceinline__ bool both_zero(double x, double y) {
    return ((unsigned long long)(bits(x) | bits(y)) << 1) == 0ull;
  }
  static __device__ __forceinline__ bool lt(double x, double y) { return key(x) < key(y) && !both_zero(x, y); }
  static __device__ __forceinline__ bool gt(double x, double y) { return key(x) > key(y) && !both_zero(x, y); }
  static __device__ __forceinline__ bool gt0(double x) { return bits(x) > 0; }
  static __device__ __forceinline__ bool lt0(double x) {
    return (unsigned long long)bits(x) > 0x8000000000000000ull;
  }
  // |x| < k and |x| >= k for k >= 0.
  static __device__ __forceinline__ bool abs_lt(double x, double k) {
    return (unsigned long long)(bits(x) & 0x7fffffffffffffffll) < (unsigned long long)bits(k);
  }
  static __device__ __forceinline__ bool is_zero(double x) { return (bits(x) << 1) == 0ll; }
  // Julia's max/min: -0.0 < +0.0.
  static __device__ __forceinline__ double max(double x, double y) { return key(x) > key(y) ? x : y; }
  static __device__ __forceinline__ double min(double x, double y) { return key(x) < key(y) ? x : y; }
#if VF_FP64_FAITHFUL
  // Reciprocal: the hardware approximation r0 (rcp.approx.ftz.f64, relative
  // error e0) refined by one third-order Newton step r0 * (1 + e + e^2) with
  // e = 1 - b*r0, whose error is e0^3 plus the rounding of the last fused
  // multiply-add. Divisors on this path are normal numbers (desingularised
  // depths >= kappa/2, wave-speed spreads >= kappa, 1 - dt*S >= 1).
  static __device__ __forceinline__ double rcp(double b) {
    double r0;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r0) : "d"(b));
    const double e = fma(-b, r0, 1.0);
    return fma(r0, fma(e, e, e), r0);
  }
  // a/b as q = a * (1/b) corrected once by the exact residual a - b*q.
  static __device__ __forceinline__ double div(double a, double b) {
    const double r = rcp(b);
    const double q = a * r;
    return fma(fma(-b, q, a), r, q);
  }
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
  struct Recip {
    double r;
  };
  static __device__ __forceinline__ Recip recip(double b) { return Recip{rcp(b)}; }
  static __device__ __forceinline__ double div_by(const Recip& R, double a) { return a * R.r; }
  static __device__ __forceinline__ double inv(const Recip& R) { return R.r; }
#elif VF_FP64_MARKSTEIN
  // Correctly rounded quotients through a correctly rounded reciprocal
  // (Markstein, IBM J. Res. Dev. 34(1), 1990; Cornea, Harrison & Tang,
  // Scientific Computing on Itanium-based Systems, ch. 8):
  //  1. y1 = the hardware reciprocal refined by one third-order Newton step,
  //     within one ulp of 1/b;
  //  2. y = y1 + y1*(1 - b*y1) (two fused multiply-adds) is RN(1/b) for every b
  //     whose significand is not all ones;
  //  3. q0 = RN(a*y) is within one ulp of a/b, the residual a - b*q0 is exact
  //     in one fused multiply-add, and RN(q0 + (a - b*q0)*y) is RN(a/b).
  // The steps need normal operands with quotients far from overflow and
  // underflow: a divisor with an all-ones significand or an exponent outside
  // +-500 (zero, subnormal, infinite and NaN divisors included), or a nonzero
  // numerator outside that range (infinite and NaN numerators included),
  // takes the IEEE division. A zero numerator over an in-range divisor
  // returns a*y, the correctly signed zero.
  struct Recip {
    double b, y;
    bool ok;
  };
  static __device__ __forceinline__ bool mid_range(long long x) {
    const int e = (int)((x >> 52) & 0x7ff);
    return e > 1023 - 500 && e < 1023 + 500;
  }
  static __device__ __forceinline__ Recip recip(double b) {
    const long long bb = bits(b);
    double r0;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r0) : "d"(b));
    const double e0 = fma(-b, r0, 1.0);
    const double y1 = fma(r0, fma(e0, e0, e0), r0);
    const double e1 = fma(-b, y1, 1.0);
    return Recip{b, fma(y1, e1, y1), mid_range(bb) && (bb & 0xfffffffffffffll) != 0xfffffffffffffll};
  }
  static __device__ __forceinline__ double div_by(const Recip& R, double a) {
    if (!R.ok) return a / R.b;
    const double q0 = a * R.y;
    if (is_zero(a)) return q0;
    if (!mid_range(bits(a))) return a / R.b;
    return fma(fma(-R.b, q0, a), R.y, q0);
  }
  static __device__ __forceinline__ double div(double a, double b) { return div_by(recip(b), a); }
  static __device__ __forceinline__ double rcp(double b) { return div(1.0, b); }
  // 1/b for terms that need no correct rounding (the derivative parts of
  // dual numbers): the correctly rounded reciprocal, where the method applies.
  static __device__ __forceinline__ double inv(const Recip& R) { return R.ok ? R.y : 1.0 / R.b; }
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
#else
  // Correctly rounded division and square root on the FP64 pipe, one IEEE
  // division per quotient. (Measured on the 4096^2 wet/dry step and not kept:
  // a correctly rounded division on the integer pipe, 40.0 vs 31.5 ms per
  // step, and quotients sharing one refined reciprocal with a Float64 rounding
  // test and a fallback, 41.1 vs 31.0 ms.)
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ double rcp(double b) { return 1.0 / b; }
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
  struct Recip {
    double b;
  };
  static __device__ __forceinline__ Recip recip(double b) { return Recip{b}; }
  static __device__ __forceinline__ double div_by(const Recip& R, double a) { return a / R.b; }
  static __device__ __forceinline__ double inv(const Recip& R) { return 1.0 / R.b; }
#endif  // VF_FP64_FAITHFUL
};

template <>
struct Arith<float> {
  static constexpr bool exact = false;
  static __device__ __forceinline__ bool lt(float x, float y) { return x < y; }
  static __device__ __forceinline__ bool gt(float x, float y) { return x > y; }
  static __device__ __forceinline__ bool gt0(float x) { return x > 0.f; }
  static __device__ __forceinline__ bool lt0(float x) { return x < 0.f; }
  static __device__ __forceinline__ bool abs_lt(float x, float k) { return fabsf(x) < k; }
  static __device__ __forceinline__ bool is_zero(float x) { return x == 0.f; }
  static __device__ __forceinline__ float max(float x, float y) { return fmaxf(x, y); }
  static __device__ __forceinline__ float min(float x, float y) { return fminf(x, y); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
  static __device__ __forceinline__ float rcp(float b) { return __fdividef(1.0f, b); }
  static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
  // Quotients over one divisor: one reciprocal, then products.
  struct Recip {
    float r;
  };
  static __device__ __forceinline__ Recip recip(float b) { return Recip{rcp(b)}; }
  static __device__ __forceinline__ float div_by(const Recip& R, float a) { return a * R.r; }
  static __device__ __forceinline__ float inv(const Recip& R) { return R.r; }
};

// ---------------------------------------------------------------------------
// Correctly rounded cube root (Float64). A libm seed is corrected with an exact
// integer comparison against the rounding midpoints, so the result is the
// nearest double regardless of the seed's last-bit error; the CPU oracle
// computes the same unique value.
__device__ __forceinline__ void cube_u55(uint64_t k, uint64_t& w0, uint64_t& w1, uint64_t& w2) {
  const uint64_t lo = k * k, hi = __umul64hi(k, k);       // k^2 < 2^110
  const uint64_t p0lo = k * lo, p0hi = __umul64hi(k, lo);  // k*lo < 2^119
  const uint64_t p1lo = k * hi, p1hi = __umul64hi(k, hi);  // k*hi < 2^101
  w0 = p0lo;
  w1 = p0hi + p1lo;
  w2 = p1hi + (w1 < p1lo ? 1ull : 0ull);
}
__device__ __forceinline__ int cmp192(uint64_t a0, uint64_t a1, uint64_t a2, uint64_t b0, uint64_t b1, uint64_t b2) {
  if (a2 != b2) return a2 < b2 ? -1 : 1;
  if (a1 != b1) return a1 < b1 ? -1 : 1;
  if (a0 != b0) return a0 < b0 ? -1 : 1;
  return 0;
}

// Out of line: the friction law calls it from two places per cell and step
// (inlined it measured 31.06 vs 31.00 ms per 4096^2 wet/dry step).
static __device__ __noinline__ double cr_cbrt(double x) {
  if (x == 0.0 || !isfinite(x)) return x;
  const bool neg = signbit(x);
  double a = fabs(x);
  int extra = 0;
  uint64_t bits = (uint64_t)__double_as_longlong(a);
  if ((bits >> 52) == 0) {
    a = a * 18014398509481984.0;  // 2^54, exact
    bits = (uint64_t)__double_as_longlong(a);
    extra = 18;
  }
  const int e = (int)(bits >> 52) - 1023;
  const uint64_t frac = bits & ((1ull << 52) - 1);
  const uint64_t M = frac | (1ull << 52);
  const int q = e >= 0 ? e / 3 : -((-e + 2) / 3);
  const int r = e - 3 * q;  // 0, 1, 2
  const double t = __longlong_as_double((long long)(((uint64_t)(1023 + r) << 52) | frac));  // in [1, 8)
  const double y0 = cbrt(t);
  uint64_t Y;
  if (y0 >= 2.0) {
    Y = 1ull << 53;
  } else if (y0 < 1.0) {
    Y = 1ull << 52;
  } else {
    Y = ((uint64_t)__double_as_longlong(y0) & ((1ull << 52) - 1)) | (1ull << 52);
  }
  // t * 2^159 = M * 2^(r + 107): limbs (0, M << (43 + r), M >> (21 - r)).
  const uint64_t T1 = M << (43 + r), T2 = M >> (21 - r);
  for (int it = 0; it < 8; ++it) {
    uint64_t c0, c1, c2;
    cube_u55(2 * Y + 1, c0, c1, c2);
    if (cmp192(c0, c1, c2, 0, T1, T2) < 0) { ++Y; continue; }
    if (Y > (1ull << 52)) {
      cube_u55(2 * Y - 1, c0, c1, c2);
      if (cmp192(c0, c1, c2, 0, T1, T2) > 0) { --Y; continue; }
    }
    break;
  }
  // y = Y * 2^(q - 52 - extra), Y in [2^52, 2^53].
  int ex = q - extra;
  uint64_t mant = Y;
  if (mant == (1ull << 53)) { mant >>= 1; ex += 1; }
  const double y = __longlong_as_double((long long)(((uint64_t)(ex + 1023) << 52) | (mant & ((1ull << 52) - 1))));
  return neg ? -y : y;
}

template <typename T> __device__ __forceinline__ T vcbrt(T x);
#if VF_FP64_FAITHFUL
template <> __device__ __forceinline__ double vcbrt<double>(double x) { return cbrt(x); }
#else
template <> __device__ __forceinline__ double vcbrt<double>(double x) { return cr_cbrt(x); }
#endif
template <> __device__ __forceinline__ float vcbrt<float>(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(__log2f(fabsf(x)) * (1.0f / 3.0f)));
  return copysignf(y, x);
}

// Back-compat names used by the tile kernels.
template <typename T> __device__ __forceinline__ T jmax(T x, T y) { return Arith<T>::max(x, y); }
template <typename T> __device__ __forceinline__ T jmin(T x, T y) { return Arith<T>::min(x, y); }
template <typename T> __device__ __forceinline__ T vdiv(T a, T b) { return Arith<T>::div(a, b); }

// ---------------------------------------------------------------------------
// Physical constants of one simulation in the state's real type.
template <typename T>
struct Phys {
  T g, neg_g, rho, c2;        // c2 = (0.5*rho)*g, as Julia folds 0.5*ρ*g*h^2
  T cutoff, kappa, theta;
  T inv_dx, inv_dy;           // 1/Δx, 1/Δy (src/numericalflux/numericalflux.jl:27)
  T dx, dy;                   // Δx, Δy (src/sourceterms/source_term_bottom.jl:38)
  int dx_pow2, dy_pow2;       // Δ is a power of two: x/Δ == x*(1/Δ) exactly
  T Cz;
  T near_dry;                 // Float32: |h| below this takes the Float64 velocity division (0: never)
  int friction;               // VF_FRICTION_*
  int n_bottom;               // SourceTermBottom entries
  int n_point;                // rain/infiltration entries, applied in order
  int rec_none;               // NoReconstruction instead of LinearReconstruction
  int any_dynamic;            // some point source is not a constant
  int point_kind[8];          // PointKind
  T point_add[8];             // kConstant: +rate/3600 for rain, -rate for infiltration
  T point_sum;                // Float32: the constant point sources' sum (summed in Float64)
  T bottom_g;                 // Float32: n_bottom * (-g), the bottom sources' factor at once
  const T* point_field[8];    // kHorton: factor, kField: rain rate [m/s]; total grid, state layout
  const double* tab_t[8];     // kTable: breakpoints of TimeDependentRain
  const double* tab_r[8];     // kTable: rates/3600 per breakpoint
  int tab_n[8];
  double horton[8][3];        // kHorton: fc, f0, k
};

enum PointKind { kConstant = 0, kTable = 1, kHorton = 2, kField = 3 };

// Deterministic exp for HortonInfiltration: Cody-Waite reduction by ln 2 (split
// in two doubles), Taylor polynomial of degree 14 in Horner form with fused
// multiply-adds, exact scaling by 2^k. The oracle computes the same bits.
__device__ __forceinline__ double det_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return __longlong_as_double(0x7ff0000000000000ll);
  if (x < -745.1332191019412) return 0.0;
  const double inv_ln2 = 0x1.71547652b82fep+0;
  const double ln2_hi = 0x1.62e42fefa39efp-1, ln2_lo = 0x1.abc9e3b39803fp-56;
  double kd = x * inv_ln2;
  kd = (kd + 6755399441055744.0) - 6755399441055744.0;  // round to nearest integer
  double r = fma(-kd, ln2_hi, x);
  r = fma(-kd, ln2_lo, r);
  const double c[15] = {0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1,
                        0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
                        0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16,
                        0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
                        0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33, 0x1.93974a8c07c9dp-37};
  double q = c[14];
#pragma unroll
  for (int n = 13; n >= 0; --n) q = fma(q, r, c[n]);
  int k = (int)kd;
  if (k > 1023) { q = q * 2.0; k -= 1; }
  if (k < -1022) return (q * __longlong_as_double((long long)(k + 54 + 1023) << 52)) * 0x1p-54;
  return q * __longlong_as_double((long long)(k + 1023) << 52);
}

// Per-step scalars of the time-dependent point sources at the step's start
// time t (the same t for both RK2 stages, src/system.jl:71-73):
// TimeDependentRain's tabulated rate (src/sourceterms/source_term_rain.jl:45-54)
// and Horton's fc + (f0 - fc)*exp(-k*t) (src/sourceterms/source_term_infiltration.jl:68-70).
template <typename T>
__device__ __forceinline__ void point_scalars(const Phys<T>& p, double t, T* out) {
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    out[n] = (T)0;
    if (n >= p.n_point) continue;
    if (p.point_kind[n] == kTable) {
      int idx = 0;
      while (idx + 1 < p.tab_n[n] && !(t < p.tab_t[n][idx + 1])) ++idx;
      out[n] = (T)p.tab_r[n][idx];
    } else if (p.point_kind[n] == kHorton) {
      const T fc = (T)p.horton[n][0], f0 = (T)p.horton[n][1], k = (T)p.horton[n][2];
      const T decay = (T)det_exp((double)(-k * (T)t));
      out[n] = fc + (f0 - fc) * decay;
    }
  }
}

// ΔB/Δ of the bottom source; exact reciprocal multiply when Δ is a power of two.
// Float32 always multiplies by 1/Δ (one rounding more where Δ is not a power
// of two; a 1.5% faster Float32 step, the same bits on power-of-two cells).
template <typename T>
__device__ __forceinline__ T slope_over(T dB, T delta, T inv_delta, int pow2) {
  if constexpr (sizeof(T) == 4) return dB * inv_delta;
  return pow2 ? dB * inv_delta : Arith<T>::div(dB, delta);
}

// Rain and infiltration in list order (src/system.jl:71-73), unrolled so the
// parameter block is never indexed dynamically. `scal` holds point_scalars();
// `cell` is the cell's offset in the state layout (for per-cell arrays).
// Float32 (the marching kernels' constant sources) adds their sum at once:
// one add instead of eight guarded ones, 2-4% of the Float32 stage pass; the
// sum rounds once to Float32 where the list order would round after each
// source (Float32 results are held to a stated error, not to the bits).
template <typename T>
__device__ __forceinline__ T add_point_sources(const Phys<T>& p, T acc0) {
  if constexpr (sizeof(T) == 4) {
    return acc0 + p.point_sum;
  } else {
#pragma unroll
    for (int n = 0; n < 8; ++n)
      if (n < p.n_point) acc0 = acc0 + p.point_add[n];
    return acc0;
  }
}
template <typename T>
__device__ __forceinline__ T add_point_sources(const Phys<T>& p, T acc0, const T* scal, long long cell) {
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    if (n >= p.n_point) continue;
    switch (p.point_kind[n]) {
      case kConstant: acc0 = acc0 + p.point_add[n]; break;
      case kTable: acc0 = acc0 + scal[n]; break;
      case kHorton: acc0 = acc0 - p.point_field[n][cell] * scal[n]; break;
      default: acc0 = acc0 + p.point_field[n][cell]; break;
    }
  }
  return acc0;
}

// desingularize, src/equations/equation.jl:40-62 (Eq. 26 of Brodtkorb & Holm 2021).
// For |h| >= kappa the expression equals h exactly: min(...) <= kappa <= |h|.
// SEL (Float32 only): the same function without a branch, the formula
// evaluated for every h (|h| >= kappa gives |h| with h's sign, i.e. h), with
// 1/(2 kappa) as a product; fewer instructions where registers allow.
template <typename T, bool SEL = false>
__device__ __forceinline__ T desing(T h, T kappa) {
  using A = Arith<T>;
  if constexpr (SEL && sizeof(T) == 4) {
    const float m = fminf(h * h * (0.5f / kappa) + kappa * 0.5f, kappa);
    return copysignf(fmaxf(fabsf(h), m), h);
  }
  if (!A::abs_lt(h, kappa)) return h;
  const T m = A::min(A::div(h * h, (T)2 * kappa) + kappa / (T)2, kappa);
  return copysign((T)1, h) * A::max(fabs(h), m);
}

// The Float64 quotient a/b of two Float32 values, rounded to Float32, without
// Float64 instructions. Rounding an IEEE quotient to 53 bits and then to 24
// gives the same bits as rounding it to 24 bits once, because 53 >= 2*24
// (Figueroa, "When is double rounding innocuous?", SIGNUM Newsl. 30(3), 1995),
// so RN32(RN64(a/b)) is the correctly rounded Float32 quotient, which
// __fdiv_rn computes on the Float32 pipes whatever the -prec-div setting. The
// kernels divide near-dry velocities with it: GB300 runs Float64 at 1/64 of
// the Float32 rate, so the Float64 instructions cost a divergent warp several
// hundred cycles per quotient. vf_selftest_near_dry_quotients checks the
// equality against the IEEE Float64 division on the device.
__device__ __forceinline__ float f64_quotient_f32(float a, float b) { return __fdiv_rn(a, b); }

// Desingularised velocities (hu, hv) / h* (src/equations/equation.jl:40-67).
// A Float32 state takes the Float64 quotient (f64_quotient_f32) where
// |h| < p.near_dry, the thin films at wet/dry fronts, and one fast reciprocal
// elsewhere; Float64 and dual numbers divide in their own type.
template <typename T>
__device__ __forceinline__ void velocities(const Phys<T>& p, T h, T hs, T hu, T hv, T& u, T& v) {
  using A = Arith<T>;
  if constexpr (sizeof(T) == 4) {
    if (A::abs_lt(h, p.near_dry)) {
      u = f64_quotient_f32(hu, hs);
      v = f64_quotient_f32(hv, hs);
      return;
    }
  }
  const typename A::Recip R = A::recip(hs);
  u = A::div_by(R, hu);
  v = A::div_by(R, hv);
}

// One side of a face: physical flux (src/equations/swe_2D.jl:43-65) and the
// two outer eigenvalues (src/equations/swe_2D.jl:69-81).
template <typename T, int DIR, bool SEL = false>
__device__ __forceinline__ void side_flux(const Phys<T>& p, T h, T hu, T hv, T& f0, T& f1, T& f2, T& l1, T& l2) {
  using A = Arith<T>;
  const T hs = desing<T, SEL>(h, p.kappa);
  T u, v;
  velocities<T>(p, h, hs, hu, hv, u, v);
  const T rh = p.rho * h;
  const T hh = h * h;
  if (DIR == 0) {
    f0 = rh * u;
    f1 = f0 * u + p.c2 * hh;
    f2 = f0 * v;
  } else {
    f0 = rh * v;
    f1 = (rh * u) * v;
    f2 = f0 * v + p.c2 * hh;
  }
  const T c = A::sqrt_(p.g * h);
  const T un = DIR == 0 ? u : v;
  l1 = un + c;
  l2 = un - c;
}

// Central-upwind flux across one face, src/numericalflux/swe/centralupwind.jl:48-77.
// minus = right face value of the left cell, plus = left face value of the right cell.
template <typename T, int DIR, bool SPEED, bool SEL = false>
__device__ __forceinline__ void cu_face(const Phys<T>& p, T mh, T mhu, T mhv, T ph, T phu, T phv, T& F0, T& F1, T& F2,
                                        T& speed) {
  using A = Arith<T>;
  T fm0 = 0, fm1 = 0, fm2 = 0, em1 = 0, em2 = 0;
  if (A::gt(mh, p.cutoff)) side_flux<T, DIR, SEL>(p, mh, mhu, mhv, fm0, fm1, fm2, em1, em2);
  T fp0 = 0, fp1 = 0, fp2 = 0, ep1 = 0, ep2 = 0;
  if (A::gt(ph, p.cutoff)) side_flux<T, DIR, SEL>(p, ph, phu, phv, fp0, fp1, fp2, ep1, ep2);
  const T aplus = A::max(A::max(ep1, em1), (T)0);
  const T aminus = A::min(A::min(ep2, em2), (T)0);
  const T d = aplus - aminus;
  if (A::abs_lt(d, p.kappa)) {
    F0 = F1 = F2 = (T)0;
    if (SPEED) speed = (T)0;
    return;
  }
  const typename A::Recip R = A::recip(d);
  const T q = A::div_by(R, aplus * aminus);
  F0 = A::div_by(R, aplus * fm0 - aminus * fp0) + q * (ph - mh);
  F1 = A::div_by(R, aplus * fm1 - aminus * fp1) + q * (phu - mhu);
  F2 = A::div_by(R, aplus * fm2 - aminus * fp2) + q * (phv - mhv);
  if (SPEED)
    speed = (A::lt(mh, p.cutoff) && A::lt(ph, p.cutoff)) ? (T)0 : A::max(fabs(aplus), fabs(aminus));
}

// minmod and minmod_slope, src/reconstruction/linearreconstruction.jl:28-43.
template <typename T>
__device__ __forceinline__ T minmod(T a, T b, T c) {
  using A = Arith<T>;
  if (A::gt0(a) && A::gt0(b) && A::gt0(c)) return A::min(A::min(a, b), c);
  if (A::lt0(a) && A::lt0(b) && A::lt0(c)) return A::max(A::max(a, b), c);
  return (T)0;
}
// Float32: the same function as max(min(a, b, c), 0) + min(max(a, b, c), 0),
// six min/max and an add instead of six compares and selects (the Float32
// kernels are instruction-issue bound: 1.007 instead of 1.083 ms per 4096^2
// wet/dry step, the same error against Float64). Float64 keeps the
// reference's branches on bit patterns.
template <>
__device__ __forceinline__ float minmod<float>(float a, float b, float c) {
  return fmaxf(fminf(fminf(a, b), c), 0.f) + fminf(fmaxf(fmaxf(a, b), c), 0.f);
}
template <typename T>
__device__ __forceinline__ T minmod_slope(T l, T c, T r, T theta) {
  const T fwd = r - c;
  const T bwd = c - l;
  const T central = (fwd + bwd) * (T)0.5;  // x/2.0 == x*0.5 exactly in binary IEEE
  return minmod<T>(theta * fwd, central, theta * bwd);
}

// Practical-SWE linear reconstruction of one cell along one direction,
// src/reconstruction/linearreconstruction.jl:73-100. Inputs are (w, hu, hv) at
// the left, middle and right cells; outputs are face (h, hu, hv).
template <typename T>
__device__ __forceinline__ void reconstruct_cell(const Phys<T>& p, const T l[3], const T c[3], const T r[3], T Bl, T Br,
                                                 T L[3], T R[3]) {
  using A = Arith<T>;
  T s0 = minmod_slope<T>(l[0], c[0], r[0], p.theta);
  const T s1 = minmod_slope<T>(l[1], c[1], r[1], p.theta);
  const T s2 = minmod_slope<T>(l[2], c[2], r[2], p.theta);
  const T w = c[0];
  if (A::lt(w - (T)0.5 * s0, Bl)) {
    s0 = (T)2 * (w - Bl);
  } else if (A::lt(w + (T)0.5 * s0, Br)) {
    s0 = (T)2 * (Br - w);
  }
  L[0] = (c[0] - (T)0.5 * s0) - Bl;
  R[0] = (c[0] + (T)0.5 * s0) - Br;
  L[1] = c[1] - (T)0.5 * s1;
  R[1] = c[1] + (T)0.5 * s1;
  L[2] = c[2] - (T)0.5 * s2;
  R[2] = c[2] + (T)0.5 * s2;
}

// Friction factor of ImplicitFriction for a 2D cell, src/friction.jl:30-43,62-78:
// S = law(Cz, h*, |u|) with h* = desingularize(w - B_cell) and u = (hu, hv)/h*.
// When hu and hv are both zero, S is -0 and the implicit division is by 1:
// callers may skip it (friction_active).
template <typename T>
__device__ __forceinline__ bool friction_active(T hu, T hv) {
  return !(Arith<T>::is_zero(hu) && Arith<T>::is_zero(hv));
}
template <typename T>
__device__ __forceinline__ T friction_factor(const Phys<T>& p, T w, T hu, T hv, T Bc) {
  using A = Arith<T>;
  const T h = w - Bc;
  const T hs = desing<T>(h, p.kappa);
  T u, v;
  velocities<T>(p, h, hs, hu, hv, u, v);
  const T speed = A::sqrt_(u * u + v * v);
  T denom;
  if (p.friction == 1) {          // friction_bsa2012
    denom = vcbrt<T>(hs) * hs;
  } else if (p.friction == 2) {   // friction_fcg2016
    denom = vcbrt<T>(hs) * hs * hs;
  } else {                        // friction_bh2021
    denom = hs * hs;
  }
  return A::div(-p.Cz * speed, denom);
}

// out[1:2] ./= (1 - dt*S) (src/friction.jl:77); skipped when S is zero, where
// the division is by exactly 1.
template <typename T>
__device__ __forceinline__ void apply_friction(T tdt, T S, T& hu, T& hv) {
  using A = Arith<T>;
  if (A::is_zero(S)) return;
  const T den = (T)1 - tdt * S;
  const typename A::Recip R = A::recip(den);
  hu = A::div_by(R, hu);
  hv = A::div_by(R, hv);
}

// Dry-cell clamp, src/timestepper/timestepper.jl:41-51.
template <typename T>
__device__ __forceinline__ void dry_clamp(const Phys<T>& p, T& w, T& hu, T& hv, T Bc) {
  using A = Arith<T>;
  if (A::lt(w - Bc, p.cutoff)) {
    w = A::max(w, Bc);
    hu = (T)0;
    hv = (T)0;
  }
}

}  // namespace vf
