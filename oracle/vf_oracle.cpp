/*
 * vf_oracle.cpp -- CPU oracle for VolumeFluxes.jl's practical 2D shallow-water step.
 *
 * TEST INFRASTRUCTURE ONLY: a restatement of the reference's CPU path used to
 * check the CUDA library and as the timed CPU baseline. The product library
 * never links or calls this file.
 *
 * Every pass mirrors one reference loop, in the reference's order, with the
 * reference's per-element expression order (no FMA contraction: build with
 * -ffp-contract=off). Passes that the reference runs over all cells
 * (zeroing, rain, infiltration, Euler update, RK2 average, friction, dry
 * clamp) run over all cells here too. Each face flux is evaluated twice, as in
 * src/numericalflux/numericalflux.jl:24-30. Citations are path:line within
 * the reference project; line numbers include the 20-line licence header.
 *
 * Parity pin: the reference publishes no golden fields. The oracle is pinned
 * by the reference's own known-answer tests for this path (minmod,
 * bottom-topography lookups, wall-BC mapping, lake at rest, rain
 * accumulation, infiltration drawdown, mirror symmetry), ported under tests/.
 *
 * cbrt (Manning-type friction laws) is evaluated correctly rounded; Julia's
 * cbrt is accurate to < 1 ulp, so the two agree except where Julia's result
 * is not the nearest double.
 */
#include "vf_oracle.h"

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <new>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Forward-mode dual number (value, derivative along one direction): the
// oracle instantiated on it stands in for ForwardDiff through the reference
// CPU path. Values are computed with exactly the double operations of the
// double oracle, so every branch is taken as in the double run; the
// derivative follows the taken branch (the subgradient at kinks).
struct Dual {
  double v, d;
  Dual() : v(0), d(0) {}
  Dual(double x) : v(x), d(0) {}  // NOLINT: constants and promoted inputs carry no derivative
  Dual(double x, double dx) : v(x), d(dx) {}
  explicit operator double() const { return v; }
  explicit operator float() const { return (float)v; }
};
inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator==(Dual a, Dual b) { return a.v == b.v; }
inline bool operator!=(Dual a, Dual b) { return a.v != b.v; }

// Math helpers with a Dual overload each.
inline bool vsignbit(double x) { return std::signbit(x); }
inline bool vsignbit(float x) { return std::signbit(x); }
inline bool vsignbit(Dual x) { return std::signbit(x.v); }
inline double vabs(double x) { return std::fabs(x); }
inline float vabs(float x) { return std::fabs(x); }
inline Dual vabs(Dual x) { return Dual(std::fabs(x.v), std::signbit(x.v) ? -x.d : x.d); }
inline double vsqrt(double x) { return std::sqrt(x); }
inline float vsqrt(float x) { return std::sqrt(x); }
inline Dual vsqrt(Dual x) {
  const double r = std::sqrt(x.v);
  return Dual(r, r > 0 ? x.d / (2 * r) : 0.0);
}
inline bool vsignbit(long double x) { return std::signbit(x); }
inline long double vabs(long double x) { return std::fabs(x); }
inline long double vsqrt(long double x) { return std::sqrt(x); }
inline long double vsign1(long double x) { return std::copysign(1.0L, x); }
inline double vsign1(double x) { return std::copysign(1.0, x); }
inline float vsign1(float x) { return std::copysign(1.0f, x); }
inline Dual vsign1(Dual x) { return Dual(std::copysign(1.0, x.v), 0.0); }

// Julia's IEEE min/max: NaN-propagating, and -0.0 < +0.0.
template <typename T>
inline T jl_max(T x, T y) {
  if (x != x || y != y) return x - y;
  return (x > y || (x == y && !vsignbit(x))) ? x : y;
}
template <typename T>
inline T jl_min(T x, T y) {
  if (x != x || y != y) return x - y;
  return (x < y || (x == y && vsignbit(x))) ? x : y;
}
template <typename T>
inline bool jl_max_picks_first(T x, T y) { return x > y || (x == y && !vsignbit(x)); }
template <typename T>
inline bool jl_min_picks_first(T x, T y) { return x < y || (x == y && vsignbit(x)); }

// ---------------------------------------------------------------------------
// Branch-outcome counters, test instrumentation for the gradient checks: when
// switched on, every evaluation of a branch of the path (minmod case,
// reconstruction clause, wet/dry face side, the kappa early-out and which
// operand wins the wave-speed max/min, the desingularised depth, the dry
// clamp) counts its outcome. Two runs whose counts agree took the same
// branches everywhere (up to exact swaps between cells, which do not happen in
// practice), so their loss difference is a smooth difference quotient; runs
// whose counts differ crossed a kink. Off by default; the counting adds one
// predictable test per branch.
enum BranchId {
  kBrMinmodMin, kBrMinmodMax, kBrMinmodZero, kBrRecLeft, kBrRecRight, kBrFaceMinusWet, kBrFacePlusWet, kBrFaceKappa,
  kBrAplusP, kBrAplusM, kBrAplusZero, kBrAminusP, kBrAminusM, kBrAminusZero, kBrDesing, kBrClamp, kBrCount
};
struct BranchCounts {
  uint64_t c[kBrCount];
};
bool g_branch_on = false;
std::mutex g_branch_mu;
std::vector<BranchCounts*> g_branch_all;  // one block per thread that counted
thread_local BranchCounts* tl_branch = nullptr;
inline void branch(int id) {
  if (!g_branch_on) return;
  if (!tl_branch) {
    tl_branch = new BranchCounts();
    std::memset(tl_branch->c, 0, sizeof(tl_branch->c));
    std::lock_guard<std::mutex> lock(g_branch_mu);
    g_branch_all.push_back(tl_branch);
  }
  ++tl_branch->c[id];
}

// ---------------------------------------------------------------------------
// Correctly rounded cube root of a double. A libm seed is corrected by an
// exact integer test on the rounding midpoints, so the result is the unique
// nearest double whatever the seed's last-bit error.
struct U192 { uint64_t w[3]; };  // w[0] least significant

inline int cmp192(const U192& a, const U192& b) {
  for (int i = 2; i >= 0; --i) {
    if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
  }
  return 0;
}

inline U192 cube_u54(uint64_t k) {  // k < 2^55
  unsigned __int128 sq = (unsigned __int128)k * k;             // < 2^110
  uint64_t lo = (uint64_t)sq, hi = (uint64_t)(sq >> 64);
  unsigned __int128 p0 = (unsigned __int128)k * lo;             // < 2^119
  unsigned __int128 p1 = (unsigned __int128)k * hi;             // < 2^101
  U192 r;
  r.w[0] = (uint64_t)p0;
  unsigned __int128 mid = (p0 >> 64) + (unsigned __int128)(uint64_t)p1;
  r.w[1] = (uint64_t)mid;
  r.w[2] = (uint64_t)(mid >> 64) + (uint64_t)(p1 >> 64);
  return r;
}

inline U192 shl192(uint64_t m, int s) {  // m << s, 64 <= s < 128
  U192 r;
  r.w[0] = 0;
  int t = s - 64;
  r.w[1] = t == 0 ? m : (m << t);
  r.w[2] = t == 0 ? 0 : (m >> (64 - t));
  return r;
}

double cr_cbrt(double x) {
  if (x == 0.0 || !std::isfinite(x)) return x;
  const bool neg = std::signbit(x);
  double a = std::fabs(x);
  int extra = 0;  // result is scaled by 2^-extra
  uint64_t bits;
  std::memcpy(&bits, &a, 8);
  if ((bits >> 52) == 0) {  // subnormal: scale by 2^54 (exact), result by 2^-18
    a = a * 18014398509481984.0;
    std::memcpy(&bits, &a, 8);
    extra = 18;
  }
  int e = (int)(bits >> 52) - 1023;
  uint64_t M = (bits & ((1ull << 52) - 1)) | (1ull << 52);
  int q = e >= 0 ? e / 3 : -((-e + 2) / 3);
  int r = e - 3 * q;                          // 0, 1, 2
  double t = std::ldexp((double)M, r - 52);  // exact, in [1, 8)
  double y0 = std::cbrt(t);
  uint64_t Y;
  if (y0 >= 2.0) {
    Y = 1ull << 53;
  } else if (y0 < 1.0) {
    Y = 1ull << 52;
  } else {
    uint64_t yb;
    std::memcpy(&yb, &y0, 8);
    Y = (yb & ((1ull << 52) - 1)) | (1ull << 52);
  }
  // cbrt(t) lies in [(2Y-1)/2^53, (2Y+1)/2^53) iff (2Y-1)^3 <= t*2^159 < (2Y+1)^3;
  // t*2^159 = M * 2^(r+107). Odd cubes never equal it, so there are no ties.
  const U192 T = shl192(M, r + 107);
  for (int it = 0; it < 8; ++it) {
    if (cmp192(cube_u54(2 * Y + 1), T) < 0) { ++Y; continue; }
    if (Y > (1ull << 52) && cmp192(cube_u54(2 * Y - 1), T) > 0) { --Y; continue; }
    break;
  }
  double y = std::ldexp((double)Y, q - 52 - extra);
  return neg ? -y : y;
}

inline float cr_cbrt(float x) { return (float)cr_cbrt((double)x); }
// Extended precision (the finite-difference reference of the gradient checks):
// the library cube root, accurate to about one ulp of long double.
inline long double cr_cbrt(long double x) { return std::cbrt(x); }
inline Dual cr_cbrt(Dual x) {
  const double r = cr_cbrt(x.v);
  return Dual(r, x.v != 0 ? x.d * r / (3 * x.v) : 0.0);
}

// ---------------------------------------------------------------------------
// Deterministic exp for HortonInfiltration: Cody-Waite reduction by ln 2 (split
// in two doubles), Taylor polynomial of degree 14 in Horner form with fused
// multiply-adds, exact scaling by 2^k. Only IEEE-exact operations, so the
// device computes the same bits. Accurate to about one ulp of Julia's exp.
double det_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return std::numeric_limits<double>::infinity();
  if (x < -745.1332191019412) return 0.0;
  const double inv_ln2 = 0x1.71547652b82fep+0;
  const double ln2_hi = 0x1.62e42fefa39efp-1, ln2_lo = 0x1.abc9e3b39803fp-56;
  double kd = x * inv_ln2;
  kd = (kd + 6755399441055744.0) - 6755399441055744.0;  // round to nearest integer
  double r = std::fma(-kd, ln2_hi, x);
  r = std::fma(-kd, ln2_lo, r);
  static const double c[15] = {0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1,
                               0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
                               0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16,
                               0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
                               0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33, 0x1.93974a8c07c9dp-37};
  double p = c[14];
  for (int n = 13; n >= 0; --n) p = std::fma(p, r, c[n]);
  int k = (int)kd;
  // p * 2^k with one rounding at most (only for subnormal results)
  if (k > 1023) { p = p * 2.0; k -= 1; }
  if (k < -1022) {
    const uint64_t b = (uint64_t)(k + 54 + 1023) << 52;
    double s1;
    std::memcpy(&s1, &b, 8);
    return (p * s1) * 0x1p-54;
  }
  const uint64_t b = (uint64_t)(k + 1023) << 52;
  double s2;
  std::memcpy(&s2, &b, 8);
  return p * s2;
}

// ---------------------------------------------------------------------------
template <typename T>
struct Sim {
  vfo_params p;
  int N1, N2;          // total cells per direction
  size_t plane;        // N1*N2
  double dx, dy;       // grid spacing, Float64 as in src/grid.jl:82-90
  std::vector<T> B;    // corners (N1+1)*(N2+1), in the real type
  // State buffers U[0..nsub]; left/right face buffers; wavespeed scalar field.
  std::vector<std::vector<T>> U;
  std::vector<T> left, right, ws;
  std::vector<double> src_times[VFO_MAX_SOURCES], src_rates[VFO_MAX_SOURCES];
  std::vector<T> src_field[VFO_MAX_SOURCES];  // Horton factor or rain field, total grid
  double t;
  double current_dt;
  double force_dt = -1;  // >= 0: every step uses this dt (frozen dt sequence)
  // Equation constants in the state's real type.
  T g, rho, cutoff, kappa, theta, cfl, Cz;

  size_t id(int i, int j) const { return (size_t)i + (size_t)N1 * (size_t)j; }
};

template <typename T>
struct Ops {
  Sim<T>& s;
  explicit Ops(Sim<T>& sim) : s(sim) {}

  // --- bottom topography lookups, src/bottom_topography.jl:86-101 ----------
  // 0-based cell (i, j) uses 0-based corners (i..i+1, j..j+1).
  T Bc(int i, int j) const {
    if (s.p.bottom_is_constant) return (T)s.p.bottom_constant;
    const int W = s.N1 + 1;
    const T* B = s.B.data();
    return (T)0.25 * (((B[i + W * j] + B[i + 1 + W * j]) + B[i + W * (j + 1)]) + B[i + 1 + W * (j + 1)]);
  }
  T Bl(int i, int j, int dir) const {
    if (s.p.bottom_is_constant) return (T)s.p.bottom_constant;
    const int W = s.N1 + 1;
    const T* B = s.B.data();
    if (dir == 0) return (T)0.5 * (B[i + W * j] + B[i + W * (j + 1)]);
    return (T)0.5 * (B[i + W * j] + B[i + 1 + W * j]);
  }
  T Br(int i, int j, int dir) const {
    if (s.p.bottom_is_constant) return (T)s.p.bottom_constant;
    const int W = s.N1 + 1;
    const T* B = s.B.data();
    if (dir == 0) return (T)0.5 * (B[i + 1 + W * j] + B[i + 1 + W * (j + 1)]);
    return (T)0.5 * (B[i + W * (j + 1)] + B[i + 1 + W * (j + 1)]);
  }

  // --- src/equations/equation.jl:40-67 -------------------------------------
  T desing(T h) const {
    const T k = s.kappa;
    T m = jl_min<T>(h * h / ((T)2 * k) + k / (T)2.0, k);
    if (g_branch_on && !jl_max_picks_first<T>(vabs(h), m)) branch(kBrDesing);
    return vsign1(h) * jl_max<T>(vabs(h), m);
  }

  // --- src/equations/swe_2D.jl:43-65 ---------------------------------------
  void phys_flux(int dir, const T* q, T* F) const {
    const T h = q[0];
    const T u = q[1] / desing(h);
    const T v = q[2] / desing(h);
    const T rho = s.rho, g = s.g;
    const T hh = h * h;
    if (dir == 0) {
      F[0] = rho * h * u;
      F[1] = rho * h * u * u + (T)0.5 * rho * g * hh;
      F[2] = rho * h * u * v;
    } else {
      F[0] = rho * h * v;
      F[1] = rho * h * u * v;
      F[2] = rho * h * v * v + (T)0.5 * rho * g * hh;
    }
  }
  // --- src/equations/swe_2D.jl:69-81 ---------------------------------------
  void eigen(int dir, const T* q, T* e) const {
    const T h = q[0];
    const T u = (dir == 0 ? q[1] : q[2]) / desing(h);
    e[0] = u + vsqrt(s.g * h);
    e[1] = u - vsqrt(s.g * h);
    e[2] = u;
  }

  // --- src/numericalflux/swe/centralupwind.jl:48-77 ------------------------
  T central_upwind(const T* fminus, const T* fplus, int dir, T* F) const {
    T flm[3] = {0, 0, 0}, em[3] = {0, 0, 0};
    if (fminus[0] > s.cutoff) {
      branch(kBrFaceMinusWet);
      phys_flux(dir, fminus, flm);
      eigen(dir, fminus, em);
    }
    T flp[3] = {0, 0, 0}, ep[3] = {0, 0, 0};
    if (fplus[0] > s.cutoff) {
      branch(kBrFacePlusWet);
      phys_flux(dir, fplus, flp);
      eigen(dir, fplus, ep);
    }
    const T aplus = jl_max<T>(jl_max<T>(ep[0], em[0]), (T)0);
    const T aminus = jl_min<T>(jl_min<T>(ep[1], em[1]), (T)0);
    if (g_branch_on) {
      const T a1 = jl_max<T>(ep[0], em[0]), b1 = jl_min<T>(ep[1], em[1]);
      branch(!jl_max_picks_first<T>(a1, (T)0) ? kBrAplusZero
                                              : jl_max_picks_first<T>(ep[0], em[0]) ? kBrAplusP : kBrAplusM);
      branch(!jl_min_picks_first<T>(b1, (T)0) ? kBrAminusZero
                                              : jl_min_picks_first<T>(ep[1], em[1]) ? kBrAminusP : kBrAminusM);
    }
    if (vabs(aplus - aminus) < s.kappa) {
      branch(kBrFaceKappa);
      F[0] = F[1] = F[2] = 0;
      return 0;
    }
    for (int k = 0; k < 3; ++k) {
      F[k] = (aplus * flm[k] - aminus * flp[k]) / (aplus - aminus) +
             ((aplus * aminus) / (aplus - aminus)) * (fplus[k] - fminus[k]);
    }
    if (fminus[0] < s.cutoff && fplus[0] < s.cutoff) return 0;
    return jl_max<T>(vabs(aplus), vabs(aminus));
  }

  // --- src/reconstruction/linearreconstruction.jl:28-43 --------------------
  static T minmod(T a, T b, T c) {
    if (a > 0 && b > 0 && c > 0) {
      branch(kBrMinmodMin);
      return jl_min<T>(jl_min<T>(a, b), c);
    }
    if (a < 0 && b < 0 && c < 0) {
      branch(kBrMinmodMax);
      return jl_max<T>(jl_max<T>(a, b), c);
    }
    branch(kBrMinmodZero);
    return 0;
  }
  static T minmod_slope(T l, T c, T r, T theta) {
    const T fwd = r - c;
    const T bwd = c - l;
    const T central = (fwd + bwd) / (T)2.0;
    return minmod(theta * fwd, central, theta * bwd);
  }

  // Buffer access: plane k of a 3-plane array.
  T& at(std::vector<T>& a, int k, int i, int j) const { return a[(size_t)k * s.plane + s.id(i, j)]; }
  T at(const std::vector<T>& a, int k, int i, int j) const { return a[(size_t)k * s.plane + s.id(i, j)]; }

  // --- src/reconstruction/linearreconstruction.jl:58-102 -------------------
  // for_each_inner_cell(...; ghostcells=1): along dir, cells 1..N-2 (0-based);
  // across, the interior (src/grid.jl:213-244).
  // --- src/reconstruction/noreconstruction.jl:30-46 ------------------------
  void reconstruct_none(const std::vector<T>& Uin) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < s.N2; ++j) {
      for (int i = 0; i < s.N1; ++i) {
        for (int k = 0; k < 3; ++k) {
          at(s.left, k, i, j) = at(Uin, k, i, j);
          at(s.right, k, i, j) = at(Uin, k, i, j);
        }
      }
    }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < s.N2; ++j) {
      for (int i = 0; i < s.N1; ++i) {
        at(s.left, 0, i, j) = at(Uin, 0, i, j) - Bc(i, j);
        at(s.right, 0, i, j) = at(Uin, 0, i, j) - Bc(i, j);
      }
    }
  }

  void reconstruct(const std::vector<T>& Uin, int dir) {
    if (s.p.reconstruction == VFO_REC_NONE) {
      reconstruct_none(Uin);
      return;
    }
    const int gc = s.p.gc;
    const int ilo = dir == 0 ? 1 : gc, ihi = dir == 0 ? s.N1 - 1 : gc + s.p.nx;
    const int jlo = dir == 0 ? gc : 1, jhi = dir == 0 ? gc + s.p.ny : s.N2 - 1;
    const int di = dir == 0 ? 1 : 0, dj = dir == 0 ? 0 : 1;
#pragma omp parallel for schedule(static)
    for (int j = jlo; j < jhi; ++j) {
      for (int i = ilo; i < ihi; ++i) {
        T slope[3];
        for (int k = 0; k < 3; ++k)
          slope[k] = minmod_slope(at(Uin, k, i - di, j - dj), at(Uin, k, i, j), at(Uin, k, i + di, j + dj), s.theta);
        const T B_left = Bl(i, j, dir);
        const T B_right = Br(i, j, dir);
        const T w = at(Uin, 0, i, j);
        if (w - (T)0.5 * slope[0] < B_left) {
          branch(kBrRecLeft);
          slope[0] = (T)2.0 * (w - B_left);
        } else if (w + (T)0.5 * slope[0] < B_right) {
          branch(kBrRecRight);
          slope[0] = (T)2.0 * (B_right - w);
        }
        for (int k = 0; k < 3; ++k) {
          at(s.left, k, i, j) = at(Uin, k, i, j) - (T)0.5 * slope[k];
          at(s.right, k, i, j) = at(Uin, k, i, j) + (T)0.5 * slope[k];
        }
        at(s.left, 0, i, j) = at(s.left, 0, i, j) - B_left;
        at(s.right, 0, i, j) = at(s.right, 0, i, j) - B_right;
      }
    }
  }

  // --- src/numericalflux/numericalflux.jl:21-33 ----------------------------
  T compute_flux(std::vector<T>& out, int dir) {
    const int gc = s.p.gc;
    const double delta = dir == 0 ? s.dx : s.dy;
    const T inv = (T)(1 / delta);
    const int di = dir == 0 ? 1 : 0, dj = dir == 0 ? 0 : 1;
#pragma omp parallel for schedule(static)
    for (int j = gc; j < gc + s.p.ny; ++j) {
      for (int i = gc; i < gc + s.p.nx; ++i) {
        T rm[3], lr[3], rl[3], lm[3];
        for (int k = 0; k < 3; ++k) {
          rm[k] = at(s.right, k, i, j);
          lr[k] = at(s.left, k, i + di, j + dj);
          rl[k] = at(s.right, k, i - di, j - dj);
          lm[k] = at(s.left, k, i, j);
        }
        T Fr[3], Fl[3];
        const T sr = central_upwind(rm, lr, dir, Fr);
        const T sl = central_upwind(rl, lm, dir, Fl);
        for (int k = 0; k < 3; ++k) at(out, k, i, j) = at(out, k, i, j) - inv * (Fr[k] - Fl[k]);
        s.ws[s.id(i, j)] = jl_max<T>(sr, sl);
      }
    }
    // maximum(wavespeeds) over the whole buffer; ghost entries stay 0.
    T m = s.ws[0];
    for (size_t n = 1; n < s.plane; ++n) m = jl_max<T>(m, s.ws[n]);
    return m;
  }

  // --- src/sourceterms/source_term_bottom.jl:24-41 -------------------------
  void bottom_source(std::vector<T>& out, int dir) {
    const int gc = s.p.gc;
    const T delta = (T)(dir == 0 ? s.dx : s.dy);
    const int k = dir == 0 ? 1 : 2;
#pragma omp parallel for schedule(static)
    for (int j = gc; j < gc + s.p.ny; ++j) {
      for (int i = gc; i < gc + s.p.nx; ++i) {
        const T B_right = Br(i, j, dir);
        const T B_left = Bl(i, j, dir);
        const T hr = at(s.right, 0, i, j), hl = at(s.left, 0, i, j);
        at(out, k, i, j) = at(out, k, i, j) + -s.g * ((B_right - B_left) / delta) * ((hr + hl) / (T)2.0);
      }
    }
  }

  // --- src/sourceterms/source_term_rain.jl:71-76 / infiltration.jl:83-88 ---
  void add_all_cells_h(std::vector<T>& out, T value, bool subtract) {
    const size_t n = s.plane;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < (long long)n; ++c) {
      out[c] = subtract ? out[c] - value : out[c] + value;
    }
  }

  // TimeDependentRain, src/sourceterms/source_term_rain.jl:45-54
  double table_rain(int n, double t) const {
    const std::vector<double>& tt = s.src_times[n];
    const std::vector<double>& rr = s.src_rates[n];
    size_t idx = 0;
    while (idx + 1 < tt.size()) {
      if (t < tt[idx + 1]) break;
      ++idx;
    }
    return rr[idx] / 3600;
  }

  // HortonInfiltration, src/sourceterms/source_term_infiltration.jl:68-70,83-88
  void horton(std::vector<T>& out, int n, double t) {
    const T fc = (T)s.p.source_rate[n], f0 = (T)s.p.source_aux[n][0], k = (T)s.p.source_aux[n][1];
    const T decay = (T)det_exp((double)(-k * (T)t));  // constants only: no derivative
    const T rate = fc + (f0 - fc) * decay;
    const std::vector<T>& f = s.src_field[n];
    const size_t m = s.plane;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < (long long)m; ++c) out[c] = out[c] - f[c] * rate;
  }

  // FunctionalRain evaluated at cell centres by the caller, source_term_rain.jl:65-76
  void rain_field(std::vector<T>& out, int n) {
    const std::vector<T>& f = s.src_field[n];
    const size_t m = s.plane;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < (long long)m; ++c) out[c] = out[c] + f[c];
  }

  // --- src/system.jl:62-75 -------------------------------------------------
  void add_time_derivative(std::vector<T>& out, const std::vector<T>& Uin, T* maxspeed, double t) {
    for (int dir = 0; dir < 2; ++dir) {
      reconstruct(Uin, dir);
      maxspeed[dir] = compute_flux(out, dir);
      for (int n = 0; n < s.p.n_sources; ++n)
        if (s.p.source_kind[n] == VFO_SRC_BOTTOM) bottom_source(out, dir);
    }
    for (int n = 0; n < s.p.n_sources; ++n) {
      switch (s.p.source_kind[n]) {
        case VFO_SRC_CONST_RAIN: add_all_cells_h(out, (T)(s.p.source_rate[n] / 3600), false); break;
        case VFO_SRC_CONST_INFIL: add_all_cells_h(out, (T)s.p.source_rate[n], true); break;
        case VFO_SRC_TIME_RAIN: add_all_cells_h(out, (T)table_rain(n, t), false); break;
        case VFO_SRC_HORTON: horton(out, n, t); break;
        case VFO_SRC_RAIN_FIELD: rain_field(out, n); break;
        default: break;
      }
    }
  }

  // --- src/friction.jl:30-43, 62-84 ----------------------------------------
  T friction_law(T c, T h, T speed) const {
    switch (s.p.friction) {
      case VFO_FRICTION_BSA2012: {
        T denom = cr_cbrt(h) * h;
        return -c * speed / denom;
      }
      case VFO_FRICTION_FCG2016: {
        T denom = cr_cbrt(h) * h * h;
        return -c * speed / denom;
      }
      default: {
        T denom = h * h;
        return -c * speed / denom;
      }
    }
  }
  void implicit_friction(std::vector<T>& out, const std::vector<T>& prev, double dt) {
    const T Cz = s.Cz;
    const T tdt = (T)dt;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < s.N2; ++j) {
      for (int i = 0; i < s.N1; ++i) {
        const T h_star = desing(at(prev, 0, i, j) - Bc(i, j));
        const T u = at(prev, 1, i, j) / h_star;
        const T v = at(prev, 2, i, j) / h_star;
        T speed = vsqrt(u * u + v * v);
        if (speed == 0) speed = 0;
        const T S = friction_law(Cz, h_star, speed);
        const T ff[3] = {(T)0, S, S};
        for (int k = 0; k < 3; ++k) at(out, k, i, j) = at(out, k, i, j) / ((T)1 - tdt * ff[k]);
      }
    }
  }

  // --- src/timestepper/timestepper.jl:41-51 --------------------------------
  void post_proc(std::vector<T>& out) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < s.N2; ++j) {
      for (int i = 0; i < s.N1; ++i) {
        const T b = Bc(i, j);
        if (at(out, 0, i, j) - b < s.cutoff) {
          branch(kBrClamp);
          at(out, 0, i, j) = jl_max<T>(at(out, 0, i, j), b);
          at(out, 1, i, j) = 0;
          at(out, 2, i, j) = 0;
        }
      }
    }
  }

  // --- src/bc.jl:29-40 -----------------------------------------------------
  void update_bc_periodic(std::vector<T>& d) {
    const int gc = s.p.gc, N1 = s.N1, N2 = s.N2;
    for (int j = gc; j < gc + s.p.ny; ++j) {
      for (int g = 1; g <= gc; ++g) {
        for (int k = 0; k < 3; ++k) {
          at(d, k, g - 1, j) = at(d, k, N1 + g - 2 * gc - 1, j);
          at(d, k, N1 - (gc - g) - 1, j) = at(d, k, gc + g - 1, j);
        }
      }
    }
    for (int g = 1; g <= gc; ++g) {
      for (int i = gc; i < gc + s.p.nx; ++i) {
        for (int k = 0; k < 3; ++k) {
          at(d, k, i, g - 1) = at(d, k, i, N2 + g - 2 * gc - 1);
          at(d, k, i, N2 - (gc - g) - 1) = at(d, k, i, gc + g - 1);
        }
      }
    }
  }

  // --- src/bc.jl:49-60: NeumannBC in 2D, as written. X: left ghosts mirror
  // the interior; on the right, data[N1-(gc-g)] = data[N1-g+1] copies ghost
  // onto ghost (g = 1, 2, ... in order). Y: bottom ghosts take the top
  // interior rows (data[i, N2+g-2gc]); on the top, ghost onto ghost again.
  // The right and top ghosts therefore keep the values the all-cell passes
  // give them.
  void update_bc_neumann(std::vector<T>& d) {
    const int gc = s.p.gc, N1 = s.N1, N2 = s.N2;
    for (int j = gc; j < gc + s.p.ny; ++j) {
      for (int g = 1; g <= gc; ++g) {
        for (int k = 0; k < 3; ++k) {
          at(d, k, g - 1, j) = at(d, k, 2 * gc - g, j);
          at(d, k, N1 - (gc - g) - 1, j) = at(d, k, N1 - g, j);
        }
      }
    }
    for (int g = 1; g <= gc; ++g) {
      for (int i = gc; i < gc + s.p.nx; ++i) {
        for (int k = 0; k < 3; ++k) {
          at(d, k, i, g - 1) = at(d, k, i, N2 + g - 2 * gc - 1);
          at(d, k, i, N2 - (gc - g) - 1) = at(d, k, i, N2 - g);
        }
      }
    }
  }

  void update_bc(std::vector<T>& d) {
    if (s.p.bc == VFO_BC_PERIODIC) update_bc_periodic(d);
    else if (s.p.bc == VFO_BC_NEUMANN) update_bc_neumann(d);
    else update_bc_wall(d);
  }

  // --- src/bc.jl:81-110 ----------------------------------------------------
  void update_bc_wall(std::vector<T>& d) {
    const int gc = s.p.gc, N1 = s.N1, N2 = s.N2;
    // X: ghost columns at interior rows.
    for (int j = gc; j < gc + s.p.ny; ++j) {
      for (int g = 1; g <= gc; ++g) {
        const int lg = g - 1, li = 2 * gc + 1 - g - 1;
        const int rg = N1 - gc + g - 1, ri = N1 - gc - g + 1 - 1;
        at(d, 0, lg, j) = at(d, 0, li, j); at(d, 1, lg, j) = -at(d, 1, li, j); at(d, 2, lg, j) = at(d, 2, li, j);
        at(d, 0, rg, j) = at(d, 0, ri, j); at(d, 1, rg, j) = -at(d, 1, ri, j); at(d, 2, rg, j) = at(d, 2, ri, j);
      }
    }
    // Y: ghost rows at interior columns.
    for (int g = 1; g <= gc; ++g) {
      const int lg = g - 1, li = 2 * gc + 1 - g - 1;
      const int rg = N2 - gc + g - 1, ri = N2 - gc - g + 1 - 1;
      for (int i = gc; i < gc + s.p.nx; ++i) {
        at(d, 0, i, lg) = at(d, 0, i, li); at(d, 1, i, lg) = at(d, 1, i, li); at(d, 2, i, lg) = -at(d, 2, i, li);
        at(d, 0, i, rg) = at(d, 0, i, ri); at(d, 1, i, rg) = at(d, 1, i, ri); at(d, 2, i, rg) = -at(d, 2, i, ri);
      }
    }
  }

  // --- src/timestepper/rungekutta.jl:26-52, forwardeuler.jl:28-47 ----------
  double do_substep(int s_idx, double dt, double max_dt) {
    std::vector<T>& out = s.U[s_idx + 1];
    const std::vector<T>& cur = s.U[s_idx];
    std::fill(out.begin(), out.end(), (T)0);
    T speed[2];
    add_time_derivative(out, cur, speed, s.t);
    if (s_idx == 0 && s.force_dt >= 0) {
      dt = s.force_dt;
    } else if (s_idx == 0) {
      // timestep_computer, src/simulator.jl:147-150
      const double dxs = s.dx / (double)speed[0];
      const double dys = s.dy / (double)speed[1];
      dt = jl_min<double>((double)s.cfl * jl_min<double>(dxs, dys), max_dt);
      if (sizeof(T) == 4) dt = (double)(float)dt;  // MVector{1,Float32} storage
    }
    const T tdt = (T)dt;
    const size_t n = 3 * s.plane;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < (long long)n; ++c) out[c] = cur[c] + tdt * out[c];
    if (s.p.stepper == VFO_STEPPER_RK2 && s_idx == 1) {
      const std::vector<T>& first = s.U[0];
#pragma omp parallel for schedule(static)
      for (long long c = 0; c < (long long)n; ++c) out[c] = (T)0.5 * (first[c] + out[c]);
    }
    return dt;
  }

  // --- src/simulator.jl:145-177 --------------------------------------------
  double perform_step(double max_dt) {
    const int nsub = s.p.stepper == VFO_STEPPER_RK2 ? 2 : 1;
    for (int st = 0; st < nsub; ++st) {
      s.current_dt = do_substep(st, s.current_dt, max_dt);
      if (s.p.friction != VFO_FRICTION_NONE) implicit_friction(s.U[st + 1], s.U[st], s.current_dt);
      post_proc(s.U[st + 1]);
      update_bc(s.U[st + 1]);
    }
    std::swap(s.U[0], s.U[nsub]);
    return s.current_dt;
  }
};

struct Handle {
  int real_bytes;
  Sim<double>* d;
  Sim<float>* f;
};

template <typename T>
Sim<T>* make_sim(const vfo_params* p, const double* Bc) {
  Sim<T>* s = new (std::nothrow) Sim<T>();
  if (!s) return nullptr;
  s->p = *p;
  s->N1 = p->nx + 2 * p->gc;
  s->N2 = p->ny + 2 * p->gc;
  s->plane = (size_t)s->N1 * s->N2;
  s->dx = (p->extent[1] - p->extent[0]) / p->nx;
  s->dy = (p->extent[3] - p->extent[2]) / p->ny;
  if (!p->bottom_is_constant) s->B.assign(Bc, Bc + (size_t)(s->N1 + 1) * (s->N2 + 1));
  const int nsub = p->stepper == VFO_STEPPER_RK2 ? 2 : 1;
  s->U.assign(nsub + 1, std::vector<T>(3 * s->plane, (T)0));
  s->left.assign(3 * s->plane, (T)0);
  s->right.assign(3 * s->plane, (T)0);
  s->ws.assign(s->plane, (T)0);
  s->t = 0;
  s->current_dt = 0;
  s->g = (T)p->g; s->rho = (T)p->rho; s->cutoff = (T)p->depth_cutoff; s->kappa = (T)p->desingularizing_kappa;
  s->theta = (T)p->theta; s->cfl = (T)p->cfl; s->Cz = (T)p->friction_Cz;
  return s;
}

int check_params(const vfo_params* p, const double* B) {
  if (!p) return -1;
  if (p->nx < 2 || p->ny < 2 || p->gc < 2) return -1;
  if (p->real_bytes != 8 && p->real_bytes != 4) return -1;
  if (p->stepper != VFO_STEPPER_FE && p->stepper != VFO_STEPPER_RK2) return -1;
  if (p->bc != VFO_BC_WALL && p->bc != VFO_BC_PERIODIC && p->bc != VFO_BC_NEUMANN) return -1;
  if (p->reconstruction != VFO_REC_LINEAR && p->reconstruction != VFO_REC_NONE) return -1;
  if (p->n_sources < 0 || p->n_sources > VFO_MAX_SOURCES) return -1;
  if (!p->bottom_is_constant && !B) return -1;
  return 0;
}

template <typename T>
void set_interior(Sim<T>* s, const double* w, const double* hu, const double* hv) {
  const double* src[3] = {w, hu, hv};
  const int gc = s->p.gc;
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < s->p.ny; ++j)
      for (int i = 0; i < s->p.nx; ++i)
        s->U[0][(size_t)k * s->plane + s->id(i + gc, j + gc)] = (T)src[k][(size_t)i + (size_t)s->p.nx * j];
  Ops<T>(*s).update_bc(s->U[0]);
}

template <typename T>
void get_interior(const Sim<T>* s, double* w, double* hu, double* hv) {
  double* dst[3] = {w, hu, hv};
  const int gc = s->p.gc;
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < s->p.ny; ++j)
      for (int i = 0; i < s->p.nx; ++i)
        dst[k][(size_t)i + (size_t)s->p.nx * j] = (double)s->U[0][(size_t)k * s->plane + s->id(i + gc, j + gc)];
}

template <typename T>
int simulate(Sim<T>* s, double endtime, int match_endtime, double maximum_timestep, long long max_steps,
             long long* steps_out) {
  Ops<T> ops(*s);
  long long n = 0;
  while (s->t < endtime) {
    double max_dt = match_endtime ? endtime - s->t : std::numeric_limits<double>::infinity();
    if (maximum_timestep >= 0) max_dt = jl_min<double>(max_dt, maximum_timestep);
    ops.perform_step(max_dt);
    if (sizeof(T) == 4)
      s->t = (double)((float)s->t + (float)s->current_dt);
    else
      s->t += s->current_dt;
    ++n;
    if (max_steps > 0 && n >= max_steps) break;
  }
  if (steps_out) *steps_out = n;
  return 0;
}

}  // namespace

extern "C" {

int vfo_create(const vfo_params* p, const double* B_corners, vfo_sim** out) {
  if (!out || check_params(p, B_corners)) return -1;
  Handle* h = new (std::nothrow) Handle();
  if (!h) return -2;
  h->real_bytes = p->real_bytes;
  h->d = nullptr;
  h->f = nullptr;
  if (p->real_bytes == 8) h->d = make_sim<double>(p, B_corners);
  else h->f = make_sim<float>(p, B_corners);
  if (!h->d && !h->f) { delete h; return -2; }
  *out = reinterpret_cast<vfo_sim*>(h);
  return 0;
}

void vfo_destroy(vfo_sim* s) {
  Handle* h = reinterpret_cast<Handle*>(s);
  if (!h) return;
  delete h->d;
  delete h->f;
  delete h;
}

int vfo_set_interior(vfo_sim* s, const double* w, const double* hu, const double* hv) {
  Handle* h = reinterpret_cast<Handle*>(s);
  if (!h || !w || !hu || !hv) return -1;
  if (h->d) set_interior(h->d, w, hu, hv); else set_interior(h->f, w, hu, hv);
  return 0;
}

int vfo_get_state(const vfo_sim* s, double* out) {
  const Handle* h = reinterpret_cast<const Handle*>(s);
  if (!h || !out) return -1;
  if (h->d) { std::memcpy(out, h->d->U[0].data(), 3 * h->d->plane * sizeof(double)); return 0; }
  for (size_t c = 0; c < 3 * h->f->plane; ++c) out[c] = (double)h->f->U[0][c];
  return 0;
}

int vfo_get_interior(const vfo_sim* s, double* w, double* hu, double* hv) {
  const Handle* h = reinterpret_cast<const Handle*>(s);
  if (!h || !w || !hu || !hv) return -1;
  if (h->d) get_interior(h->d, w, hu, hv); else get_interior(h->f, w, hu, hv);
  return 0;
}

int vfo_perform_step(vfo_sim* s, double max_dt, double* dt_out) {
  Handle* h = reinterpret_cast<Handle*>(s);
  if (!h) return -1;
  double dt = h->d ? Ops<double>(*h->d).perform_step(max_dt) : Ops<float>(*h->f).perform_step(max_dt);
  if (dt_out) *dt_out = dt;
  return 0;
}

int vfo_simulate_to_time(vfo_sim* s, double endtime, int match_endtime, double maximum_timestep,
                         long long max_steps, long long* steps_out) {
  Handle* h = reinterpret_cast<Handle*>(s);
  if (!h) return -1;
  return h->d ? simulate(h->d, endtime, match_endtime, maximum_timestep, max_steps, steps_out)
              : simulate(h->f, endtime, match_endtime, maximum_timestep, max_steps, steps_out);
}

double vfo_time(const vfo_sim* s) {
  const Handle* h = reinterpret_cast<const Handle*>(s);
  return h->d ? h->d->t : h->f->t;
}

void vfo_set_time(vfo_sim* s, double t) {
  Handle* h = reinterpret_cast<Handle*>(s);
  if (h->d) h->d->t = t; else h->f->t = t;
}

double vfo_current_timestep(const vfo_sim* s) {
  const Handle* h = reinterpret_cast<const Handle*>(s);
  return h->d ? h->d->current_dt : h->f->current_dt;
}

int vfo_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int vfo_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

double vfo_minmod(double a, double b, double c) { return Ops<double>::minmod(a, b, c); }
double vfo_minmod_slope(double l, double c, double r, double theta) {
  return Ops<double>::minmod_slope(l, c, r, theta);
}

double vfo_bottom_lookup(const double* B, int n1p1, int n2p1, int i, int j, int which) {
  (void)n2p1;
  const int W = n1p1;
  const int x = i - 1, y = j - 1;  // reference indices are 1-based
  switch (which) {
    case 0: return 0.25 * (B[x + W * y] + B[x + 1 + W * y] + B[x + W * (y + 1)] + B[x + 1 + W * (y + 1)]);
    case 1: return 0.5 * (B[x + W * y] + B[x + W * (y + 1)]);
    case 2: return 0.5 * (B[x + 1 + W * y] + B[x + 1 + W * (y + 1)]);
    case 3: return 0.5 * (B[x + W * y] + B[x + 1 + W * y]);
    case 4: return 0.5 * (B[x + W * (y + 1)] + B[x + 1 + W * (y + 1)]);
    default: return std::numeric_limits<double>::quiet_NaN();
  }
}

int vfo_update_bc_wall(double* state, int nx, int ny, int gc) {
  if (!state || nx < gc || ny < gc || gc < 1) return -1;
  Sim<double> s;
  std::memset(&s.p, 0, sizeof(s.p));
  s.p.nx = nx; s.p.ny = ny; s.p.gc = gc; s.p.bc = VFO_BC_WALL;
  s.N1 = nx + 2 * gc; s.N2 = ny + 2 * gc;
  s.plane = (size_t)s.N1 * s.N2;
  std::vector<double> d(state, state + 3 * s.plane);
  Ops<double>(s).update_bc(d);
  std::memcpy(state, d.data(), 3 * s.plane * sizeof(double));
  return 0;
}

double vfo_cbrt(double x) { return cr_cbrt(x); }

double vfo_exp(double x) { return det_exp(x); }

int vfo_set_source_table(vfo_sim* sim, int index, const double* times, const double* rates, int n) {
  Handle* h = reinterpret_cast<Handle*>(sim);
  if (!h || index < 0 || index >= VFO_MAX_SOURCES || n < 1 || !times || !rates) return -1;
  auto set = [&](auto* S) {
    S->src_times[index].assign(times, times + n);
    S->src_rates[index].assign(rates, rates + n);
  };
  if (h->d) set(h->d); else set(h->f);
  return 0;
}

int vfo_set_source_field(vfo_sim* sim, int index, const double* field) {
  Handle* h = reinterpret_cast<Handle*>(sim);
  if (!h || index < 0 || index >= VFO_MAX_SOURCES || !field) return -1;
  auto set = [&](auto* S) {
    S->src_field[index].resize(S->plane);
    for (size_t c = 0; c < S->plane; ++c) S->src_field[index][c] = (decltype(S->src_field[index][0] + 0))field[c];
  };
  if (h->d) set(h->d); else set(h->f);
  return 0;
}

int vfo_update_bc_periodic(double* state, int nx, int ny, int gc) {
  if (!state || nx < gc || ny < gc || gc < 1) return -1;
  Sim<double> s;
  std::memset(&s.p, 0, sizeof(s.p));
  s.p.nx = nx; s.p.ny = ny; s.p.gc = gc; s.p.bc = VFO_BC_PERIODIC;
  s.N1 = nx + 2 * gc; s.N2 = ny + 2 * gc;
  s.plane = (size_t)s.N1 * s.N2;
  std::vector<double> d(state, state + 3 * s.plane);
  Ops<double>(s).update_bc(d);
  std::memcpy(state, d.data(), 3 * s.plane * sizeof(double));
  return 0;
}

int vfo_update_bc_neumann(double* state, int nx, int ny, int gc) {
  if (!state || nx < gc || ny < gc || gc < 1) return -1;
  Sim<double> s;
  std::memset(&s.p, 0, sizeof(s.p));
  s.p.nx = nx; s.p.ny = ny; s.p.gc = gc; s.p.bc = VFO_BC_NEUMANN;
  s.N1 = nx + 2 * gc; s.N2 = ny + 2 * gc;
  s.plane = (size_t)s.N1 * s.N2;
  std::vector<double> d(state, state + 3 * s.plane);
  Ops<double>(s).update_bc(d);
  std::memcpy(state, d.data(), 3 * s.plane * sizeof(double));
  return 0;
}

}  // extern "C"

namespace {
// The source tables and per-cell source fields of an existing Float64
// simulation (TimeDependentRain, HortonInfiltration, a rain field), converted
// to the real type of dst.
template <typename T>
void copy_sources(Sim<T>* dst, const vfo_sim* like) {
  if (!like) return;
  const Handle* h = reinterpret_cast<const Handle*>(like);
  if (!h->d) return;
  for (int i = 0; i < VFO_MAX_SOURCES; ++i) {
    dst->src_times[i] = h->d->src_times[i];
    dst->src_rates[i] = h->d->src_rates[i];
    dst->src_field[i].assign(h->d->src_field[i].begin(), h->d->src_field[i].end());
  }
}

// From the given interior state at t = 0, n_steps steps with the frozen dt
// sequence, t += dt after each (the time of the time-dependent sources);
// loss = sum over gauges of (w - target)^2 in the simulation's type.
template <typename T>
T frozen_gauge_loss(Sim<T>* s, const double* w, const double* hu, const double* hv, const double* dts, int n_steps,
                    const int* gauge_i, const int* gauge_j, const double* target, int n_gauges) {
  set_interior(s, w, hu, hv);
  Ops<T> ops(*s);
  s->t = 0.0;
  for (int k = 0; k < n_steps; ++k) {
    s->force_dt = dts[k];
    ops.perform_step(std::numeric_limits<double>::infinity());
    s->t = s->t + dts[k];
  }
  T L(0.0);
  const int gc = s->p.gc;
  for (int g = 0; g < n_gauges; ++g) {
    const T x = s->U[0][s->id(gauge_i[g] + gc, gauge_j[g] + gc)] - T(target[g]);
    L = L + x * x;
  }
  return L;
}
}  // namespace

extern "C" {

int vfo_dual_gauge_loss(const vfo_params* p, const double* B, const double* Bdot, double Cz_dot, const double* w,
                        const double* hu, const double* hv, const double* dts, int n_steps, const int* gauge_i,
                        const int* gauge_j, const double* target, int n_gauges, double* loss, double* dloss,
                        const vfo_sim* like) {
  if (check_params(p, B) || !loss || n_steps < 0 || (n_steps > 0 && !dts) || n_gauges < 0) return -1;
  if (p->real_bytes != 8) return -1;
  Sim<Dual>* s = make_sim<Dual>(p, B);
  if (!s) return -2;
  copy_sources(s, like);
  if (Bdot && !p->bottom_is_constant)
    for (size_t c = 0; c < s->B.size(); ++c) s->B[c].d = Bdot[c];
  s->Cz.d = Cz_dot;
  const Dual L = frozen_gauge_loss<Dual>(s, w, hu, hv, dts, n_steps, gauge_i, gauge_j, target, n_gauges);
  *loss = L.v;
  if (dloss) *dloss = L.d;
  delete s;
  return 0;
}

int vfo_frozen_gauge_loss(const vfo_params* p, const double* B, const double* w, const double* hu, const double* hv,
                          const double* dts, int n_steps, const int* gauge_i, const int* gauge_j,
                          const double* target, int n_gauges, double* loss, const vfo_sim* like) {
  if (check_params(p, B) || !loss || n_steps < 0 || (n_steps > 0 && !dts) || n_gauges < 0) return -1;
  if (p->real_bytes != 8) return -1;
  Sim<double>* s = make_sim<double>(p, B);
  if (!s) return -2;
  copy_sources(s, like);
  *loss = frozen_gauge_loss<double>(s, w, hu, hv, dts, n_steps, gauge_i, gauge_j, target, n_gauges);
  delete s;
  return 0;
}

int vfo_ext_gauge_loss(const vfo_params* p, const double* B, const double* Bdir, double Cz_dir1, double Cz_dir2,
                       double eps, const double* w, const double* hu, const double* hv, const double* dts,
                       int n_steps, const int* gauge_i, const int* gauge_j, const double* target, int n_gauges,
                       double* loss_hi, double* loss_lo, const vfo_sim* like) {
  if (check_params(p, B) || !loss_hi || !loss_lo || n_steps < 0 || (n_steps > 0 && !dts) || n_gauges < 0)
    return -1;
  if (p->real_bytes != 8) return -1;
  Sim<long double>* s = make_sim<long double>(p, B);
  if (!s) return -2;
  copy_sources(s, like);
  const long double e = eps;
  if (Bdir && !p->bottom_is_constant)
    for (size_t c = 0; c < s->B.size(); ++c) s->B[c] = (long double)B[c] + e * (long double)Bdir[c];
  s->Cz = (long double)p->friction_Cz + e * (long double)Cz_dir1 + e * e * (long double)Cz_dir2;
  const long double L = frozen_gauge_loss<long double>(s, w, hu, hv, dts, n_steps, gauge_i, gauge_j, target, n_gauges);
  *loss_hi = (double)L;
  *loss_lo = (double)(L - (long double)*loss_hi);
  delete s;
  return 0;
}

void vfo_branch_counting(int on) {
  std::lock_guard<std::mutex> lock(g_branch_mu);
  for (BranchCounts* b : g_branch_all) std::memset(b->c, 0, sizeof(b->c));
  g_branch_on = on != 0;
}

int vfo_branch_counts(unsigned long long* out, int n) {
  std::lock_guard<std::mutex> lock(g_branch_mu);
  for (int i = 0; i < n && i < kBrCount; ++i) {
    unsigned long long sum = 0;
    for (BranchCounts* b : g_branch_all) sum += b->c[i];
    out[i] = sum;
  }
  return kBrCount;
}

double vfo_desingularize(double h, double kappa) {
  Sim<double> s;
  s.kappa = kappa;
  return Ops<double>(s).desing(h);
}

}  // extern "C"
