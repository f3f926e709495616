// vf_math.cuh -- per-cell and per-face arithmetic of VolumeFluxes.jl's
// practical 2D shallow-water path, restated for the device.
//
// Every expression keeps the reference's operation order, because the Float64
// path must reproduce the reference bit for bit: the Float64 translation unit
// is compiled with -fmad=false, so a*b+c stays two rounded operations as in
// Julia. Float32 instances may contract (their error is stated against the
// Float64 oracle, not claimed bitwise).
//
// Citations are path:line within the VolumeFluxes.jl project.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace vf {

// Julia's min/max on IEEE floats order -0.0 below +0.0
// (relevant when a dry face contributes +0 against a -0 eigenvalue).
// NaN operands cannot occur on a valid step (every divisor is bounded away
// from zero), so NaN ordering is not reproduced here.
template <typename T>
__device__ __forceinline__ T jmax(T x, T y) {
  return (x > y || (x == y && !signbit(x))) ? x : y;
}
template <typename T>
__device__ __forceinline__ T jmin(T x, T y) {
  return (x < y || (x == y && signbit(x))) ? x : y;
}

// Division. Float64 keeps IEEE division (bitwise parity); Float32 may use the
// fast reciprocal path.
template <typename T> __device__ __forceinline__ T vdiv(T a, T b);
template <> __device__ __forceinline__ double vdiv<double>(double a, double b) { return a / b; }
template <> __device__ __forceinline__ float vdiv<float>(float a, float b) { return __fdividef(a, b); }

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
template <> __device__ __forceinline__ double vcbrt<double>(double x) { return cr_cbrt(x); }
template <> __device__ __forceinline__ float vcbrt<float>(float x) { return cbrtf(x); }

// ---------------------------------------------------------------------------
// Physical constants of one simulation in the state's real type.
template <typename T>
struct Phys {
  T g, neg_g, rho, c2;        // c2 = (0.5*rho)*g, as Julia folds 0.5*ρ*g*h^2
  T cutoff, kappa, theta;
  T inv_dx, inv_dy;           // 1/Δx, 1/Δy (src/numericalflux/numericalflux.jl:27)
  T dx, dy;                   // Δx, Δy (src/sourceterms/source_term_bottom.jl:38)
  T Cz;
  int friction;               // VF_FRICTION_*
  int n_bottom;               // SourceTermBottom entries
  int n_point;                // rain/infiltration entries, applied in order
  T point_add[8];             // +rate/3600 for rain, -rate for infiltration
};

// desingularize, src/equations/equation.jl:40-62 (Eq. 26 of Brodtkorb & Holm 2021).
// For |h| >= kappa the expression equals h exactly: min(...) <= kappa <= |h|.
template <typename T>
__device__ __forceinline__ T desing(T h, T kappa) {
  const T ah = fabs(h);
  if (ah >= kappa) return h;
  const T m = jmin<T>(vdiv<T>(h * h, (T)2 * kappa) + kappa / (T)2, kappa);
  return copysign((T)1, h) * jmax<T>(ah, m);
}

// One side of a face: physical flux (src/equations/swe_2D.jl:43-65) and the
// two outer eigenvalues (src/equations/swe_2D.jl:69-81).
template <typename T, int DIR>
__device__ __forceinline__ void side_flux(const Phys<T>& p, T h, T hu, T hv, T& f0, T& f1, T& f2, T& l1, T& l2) {
  const T hs = desing<T>(h, p.kappa);
  const T u = vdiv<T>(hu, hs);
  const T v = vdiv<T>(hv, hs);
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
  const T c = sqrt(p.g * h);
  const T un = DIR == 0 ? u : v;
  l1 = un + c;
  l2 = un - c;
}

// Central-upwind flux across one face, src/numericalflux/swe/centralupwind.jl:48-77.
// minus = right face value of the left cell, plus = left face value of the right cell.
template <typename T, int DIR, bool SPEED>
__device__ __forceinline__ void cu_face(const Phys<T>& p, T mh, T mhu, T mhv, T ph, T phu, T phv, T& F0, T& F1, T& F2,
                                        T& speed) {
  T fm0 = 0, fm1 = 0, fm2 = 0, em1 = 0, em2 = 0;
  if (mh > p.cutoff) side_flux<T, DIR>(p, mh, mhu, mhv, fm0, fm1, fm2, em1, em2);
  T fp0 = 0, fp1 = 0, fp2 = 0, ep1 = 0, ep2 = 0;
  if (ph > p.cutoff) side_flux<T, DIR>(p, ph, phu, phv, fp0, fp1, fp2, ep1, ep2);
  const T aplus = jmax<T>(jmax<T>(ep1, em1), (T)0);
  const T aminus = jmin<T>(jmin<T>(ep2, em2), (T)0);
  const T d = aplus - aminus;
  if (fabs(d) < p.kappa) {
    F0 = F1 = F2 = (T)0;
    if (SPEED) speed = (T)0;
    return;
  }
  const T q = vdiv<T>(aplus * aminus, d);
  F0 = vdiv<T>(aplus * fm0 - aminus * fp0, d) + q * (ph - mh);
  F1 = vdiv<T>(aplus * fm1 - aminus * fp1, d) + q * (phu - mhu);
  F2 = vdiv<T>(aplus * fm2 - aminus * fp2, d) + q * (phv - mhv);
  if (SPEED) speed = (mh < p.cutoff && ph < p.cutoff) ? (T)0 : jmax<T>(fabs(aplus), fabs(aminus));
}

// minmod and minmod_slope, src/reconstruction/linearreconstruction.jl:28-43.
template <typename T>
__device__ __forceinline__ T minmod(T a, T b, T c) {
  if (a > (T)0 && b > (T)0 && c > (T)0) return jmin<T>(jmin<T>(a, b), c);
  if (a < (T)0 && b < (T)0 && c < (T)0) return jmax<T>(jmax<T>(a, b), c);
  return (T)0;
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
  T s0 = minmod_slope<T>(l[0], c[0], r[0], p.theta);
  const T s1 = minmod_slope<T>(l[1], c[1], r[1], p.theta);
  const T s2 = minmod_slope<T>(l[2], c[2], r[2], p.theta);
  const T w = c[0];
  if (w - (T)0.5 * s0 < Bl) {
    s0 = (T)2 * (w - Bl);
  } else if (w + (T)0.5 * s0 < Br) {
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
template <typename T>
__device__ __forceinline__ T friction_factor(const Phys<T>& p, T w, T hu, T hv, T Bc) {
  const T hs = desing<T>(w - Bc, p.kappa);
  const T u = vdiv<T>(hu, hs);
  const T v = vdiv<T>(hv, hs);
  const T speed = sqrt(u * u + v * v);
  T denom;
  if (p.friction == 1) {          // friction_bsa2012
    denom = vcbrt<T>(hs) * hs;
  } else if (p.friction == 2) {   // friction_fcg2016
    denom = vcbrt<T>(hs) * hs * hs;
  } else {                        // friction_bh2021
    denom = hs * hs;
  }
  return vdiv<T>(-p.Cz * speed, denom);
}

// Dry-cell clamp, src/timestepper/timestepper.jl:41-51.
template <typename T>
__device__ __forceinline__ void dry_clamp(const Phys<T>& p, T& w, T& hu, T& hv, T Bc) {
  if (w - Bc < p.cutoff) {
    w = jmax<T>(w, Bc);
    hu = (T)0;
    hv = (T)0;
  }
}

}  // namespace vf
