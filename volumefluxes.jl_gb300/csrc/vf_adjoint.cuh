// vf_adjoint.cuh -- reverse (adjoint) kernels of one RK2 step with a frozen dt.
//
// For a loss of the final state, the reverse sweep carries lambda = dLoss/dU
// backwards through every step and accumulates dLoss/dB (bottom corners) and
// dLoss/dCz (friction coefficient). One step is reversed stage by stage, each
// stage in four kernels that read the recomputed forward data:
//   k_adj_point   the stage's pointwise part in reverse: dry clamp, implicit
//                 friction (dS/d(w,hu,hv,B_cell,Cz) from dual numbers through
//                 friction_factor), RK2 average, Euler update; gives
//                 lambda of L (the stage's time derivative) and the direct
//                 lambda of the stage input;
//   k_adj_recon   per cell and direction: lambda of the cell's two face values
//                 from the central-upwind flux of each adjacent face (local
//                 Jacobians from dual numbers through cu_face) and from the
//                 bottom source, then the minmod reconstruction in reverse
//                 (the subgradient of the branch the forward pass took), split
//                 into contributions to the cell and its two neighbours;
//   k_adj_gather  lambda of the stage input per interior cell: the direct part
//                 plus the neighbour contributions, with the lambda of wall
//                 ghost cells folded onto the interior cells they mirror;
//   k_adj_corner  dLoss/dB per corner from the B_cell and face-bottom parts.
// Dual numbers evaluate the very functions of the forward kernels
// (vf_math.cuh), so their values -- and every branch -- are the forward
// pass's; the derivatives follow the branch taken (the subgradient at kinks:
// minmod switches, dry faces, the dry clamp). Gathers instead of atomics keep
// the sums in a fixed order: the gradient is deterministic.
#pragma once
#include "vf_kernels.cuh"

namespace vf {

// ---------------------------------------------------------------------------
// Forward-mode dual numbers on the device.
template <typename T>
struct Dual {
  T v, d;
  __device__ __forceinline__ Dual() : v(0), d(0) {}
  __device__ __forceinline__ Dual(T x, T dx) : v(x), d(dx) {}
  template <typename S>
  __device__ __forceinline__ Dual(S x) : v((T)x), d((T)0) {}  // constants carry no derivative
};

template <typename T>
__device__ __forceinline__ Dual<T> operator+(Dual<T> a, Dual<T> b) { return Dual<T>(a.v + b.v, a.d + b.d); }
template <typename T>
__device__ __forceinline__ Dual<T> operator-(Dual<T> a, Dual<T> b) { return Dual<T>(a.v - b.v, a.d - b.d); }
template <typename T>
__device__ __forceinline__ Dual<T> operator-(Dual<T> a) { return Dual<T>(-a.v, -a.d); }
// Derivative parts use fused multiply-adds and reciprocals where the value
// parts keep the forward pass's exact operations: values and branches stay
// the forward pass's, derivatives change at the rounding level only.
template <typename T>
__device__ __forceinline__ Dual<T> operator*(Dual<T> a, Dual<T> b) { return Dual<T>(a.v * b.v, fma(a.d, b.v, a.v * b.d)); }
template <typename T>
__device__ __forceinline__ Dual<T> operator/(Dual<T> a, Dual<T> b) {
  const T q = a.v / b.v;
  return Dual<T>(q, (a.d - q * b.d) / b.v);
}
template <typename T>
__device__ __forceinline__ Dual<T> copysign(Dual<T> a, Dual<T> b) {
  return Dual<T>(::copysign(a.v, b.v), (T)0);  // used as copysign(1, h): a constant
}
template <typename T>
__device__ __forceinline__ Dual<T> fabs(Dual<T> a) {
  return Dual<T>(::fabs(a.v), ::signbit(a.v) ? -a.d : a.d);
}

template <typename T>
struct Arith<Dual<T>> {
  using A = Arith<T>;
  using D = Dual<T>;
  static constexpr bool exact = A::exact;
  static __device__ __forceinline__ bool lt(D x, D y) { return A::lt(x.v, y.v); }
  static __device__ __forceinline__ bool gt(D x, D y) { return A::gt(x.v, y.v); }
  static __device__ __forceinline__ bool gt0(D x) { return A::gt0(x.v); }
  static __device__ __forceinline__ bool lt0(D x) { return A::lt0(x.v); }
  static __device__ __forceinline__ bool abs_lt(D x, D k) { return A::abs_lt(x.v, k.v); }
  static __device__ __forceinline__ bool is_zero(D x) { return A::is_zero(x.v); }
  // The operand the forward max/min returns, with its derivative.
  static __device__ __forceinline__ D max(D x, D y) { return picks_second_max(x.v, y.v) ? y : x; }
  static __device__ __forceinline__ D min(D x, D y) { return picks_second_min(x.v, y.v) ? y : x; }
  static __device__ __forceinline__ D div(D a, D b) {
    const T q = A::div(a.v, b.v);
    return D(q, fma(-q, b.d, a.d) * A::inv(A::recip(b.v)));
  }
  static __device__ __forceinline__ D rcp(D b) {
    const T r = A::rcp(b.v);
    return D(r, -b.d * r * r);
  }
  static __device__ __forceinline__ D sqrt_(D x) {
    const T r = A::sqrt_(x.v);
    return D(r, r > (T)0 ? x.d * ((T)0.5 * A::inv(A::recip(r))) : (T)0);
  }
  // Quotients over one divisor: values as the forward's div_by, derivatives of a/b.
  struct Recip {
    D b;
    typename A::Recip R;
  };
  static __device__ __forceinline__ Recip recip(D b) { return Recip{b, A::recip(b.v)}; }
  static __device__ __forceinline__ D div_by(const Recip& R, D a) {
    const T q = A::div_by(R.R, a.v);
    return D(q, fma(-q, R.b.d, a.d) * A::inv(R.R));
  }
  // For equal values the forward max/min may return either operand; these
  // say which, so the derivative follows the same operand.
  static __device__ __forceinline__ bool picks_second_max(T x, T y) {
    if constexpr (sizeof(T) == 8) return !(Arith<double>::key(x) > Arith<double>::key(y));
    return !(x >= y);
  }
  static __device__ __forceinline__ bool picks_second_min(T x, T y) {
    if constexpr (sizeof(T) == 8) return !(Arith<double>::key(x) < Arith<double>::key(y));
    return !(x <= y);
  }
};

template <>
__device__ __forceinline__ Dual<double> vcbrt<Dual<double>>(Dual<double> x) {
  const double r = vcbrt<double>(x.v);
  return Dual<double>(r, x.v != 0.0 ? x.d * r * Arith<double>::inv(Arith<double>::recip(3.0 * x.v)) : 0.0);
}
template <>
__device__ __forceinline__ Dual<float> vcbrt<Dual<float>>(Dual<float> x) {
  const float r = vcbrt<float>(x.v);
  return Dual<float>(r, x.v != 0.f ? x.d * r / (3.f * x.v) : 0.f);
}

// The scalars cu_face and friction_factor read, as constants of dual type.
template <typename T>
__device__ __forceinline__ Phys<Dual<T>> dual_phys(const Phys<T>& p) {
  Phys<Dual<T>> q;
  q.g = p.g;
  q.neg_g = p.neg_g;
  q.rho = p.rho;
  q.c2 = p.c2;
  q.cutoff = p.cutoff;
  q.kappa = p.kappa;
  q.theta = p.theta;
  q.inv_dx = p.inv_dx;
  q.inv_dy = p.inv_dy;
  q.dx = p.dx;
  q.dy = p.dy;
  q.dx_pow2 = p.dx_pow2;
  q.dy_pow2 = p.dy_pow2;
  q.Cz = p.Cz;
  q.near_dry = p.near_dry;
  q.friction = p.friction;
  q.n_bottom = p.n_bottom;
  q.n_point = 0;
  q.rec_none = p.rec_none;
  q.any_dynamic = 0;
  return q;
}

// ---------------------------------------------------------------------------
template <typename T>
struct AdjArgs {
  Geom<T> g;
  Phys<T> p;
  const T* B;
  double dt;
  int stage2;           // 1: the RK2 second stage (RK2 average with Ubase)
  const T* Uprev;       // the stage's input (friction and Euler update)
  const T* Ubase;       // stage 2: U^n of the RK2 average
  const T* L;           // the stage's time derivative (forward)
  const T* lam_out;     // lambda of the stage's output (interior cells)
  T* lamL;              // lambda of L (interior cells)
  T* lam_direct;        // lambda of Uprev through the pointwise part
  T* lam_base;          // lambda of U^n through the stage-2 average (written by stage 2, read by stage 1)
  T* gBc;               // dLoss/dB_cell per interior cell
  double* gCz_part;     // one partial sum per block of k_adj_point
  T* C[2];              // per direction: 9 planes = (to c-1, to c, to c+1) x (w, hu, hv)
  T* gBf[2];            // per direction: 2 planes (left face bottom, right face bottom) per cell
  T* lam_in;            // gather output: lambda of the stage input
  double* gB;           // dLoss/dB per corner, accumulated
};

template <typename T>
__device__ __forceinline__ T cell_bottom(const Geom<T>& g, const T* __restrict__ B, int x, int y) {
  if (g.bottom_const) return g.bconst;
  const long long b = (long long)y * g.PB + x + XOFF;
  return (T)0.25 * (((B[b] + B[b + 1]) + B[b + g.PB]) + B[b + g.PB + 1]);
}

// Stage pointwise part in reverse (one interior cell per thread).
template <typename T>
__global__ void __launch_bounds__(256) k_adj_point(AdjArgs<T> a) {
  using A = Arith<T>;
  __shared__ double red[256];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int x = a.g.gc + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = a.g.gc + blockIdx.y * blockDim.y + threadIdx.y;
  double gcz = 0.0;
  if (x < a.g.gc + a.g.nx && y < a.g.gc + a.g.ny) {
    const Geom<T>& g = a.g;
    const Phys<T>& p = a.p;
    const long long o = sidx(g, x, y);
    const T tdt = (T)a.dt;
    const T Bc = cell_bottom(g, a.B, x, y);
    const T q0 = a.Uprev[o], q1 = a.Uprev[g.PS + o], q2 = a.Uprev[2 * g.PS + o];
    const T l0 = a.L[o], l1 = a.L[g.PS + o], l2 = a.L[2 * g.PS + o];
    // forward, as stage1_point / the stage-2 epilogue compute it
    T w = q0 + tdt * l0, hu = q1 + tdt * l1, hv = q2 + tdt * l2;
    T b0 = 0, b1 = 0, b2 = 0;
    if (a.stage2) {
      b0 = a.Ubase[o];
      b1 = a.Ubase[g.PS + o];
      b2 = a.Ubase[2 * g.PS + o];
      w = (T)0.5 * (b0 + w);
      hu = (T)0.5 * (b1 + hu);
      hv = (T)0.5 * (b2 + hv);
    }
    T S = (T)0;
    if (p.friction && friction_active<T>(q1, q2)) S = friction_factor<T>(p, q0, q1, q2, Bc);
    const bool fric = p.friction && !A::is_zero(S);
    T den = (T)1;
    if (fric) {
      den = (T)1 - tdt * S;
      apply_friction<T>(tdt, S, hu, hv);
    }
    // reverse
    T lw = a.lam_out[o], lhu = a.lam_out[g.PS + o], lhv = a.lam_out[2 * g.PS + o];
    T gbc = (T)0;
    if (A::lt(w - Bc, p.cutoff)) {  // dry clamp: (max(w, Bc), 0, 0)
      if (Arith<Dual<T>>::picks_second_max(w, Bc)) {  // Bc kept
        gbc = gbc + lw;
        lw = (T)0;
      }
      lhu = (T)0;
      lhv = (T)0;
    }
    T lq0 = 0, lq1 = 0, lq2 = 0;
    if (fric) {
      // hu_out = huA / den, den = 1 - dt*S(Uprev, Bc, Cz)
      const T lden = -(lhu * hu + lhv * hv) / den;
      lhu = lhu / den;
      lhv = lhv / den;
      const T lS = -tdt * lden;
      const Phys<Dual<T>> dp = dual_phys(p);
      T grad[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        Phys<Dual<T>> pk = dp;
        if (k == 4) pk.Cz = Dual<T>(p.Cz, (T)1);
        const Dual<T> dw(q0, k == 0 ? (T)1 : (T)0), dhu(q1, k == 1 ? (T)1 : (T)0), dhv(q2, k == 2 ? (T)1 : (T)0);
        const Dual<T> dB(Bc, k == 3 ? (T)1 : (T)0);
        grad[k] = friction_factor<Dual<T>>(pk, dw, dhu, dhv, dB).d;
      }
      lq0 = lq0 + lS * grad[0];
      lq1 = lq1 + lS * grad[1];
      lq2 = lq2 + lS * grad[2];
      gbc = gbc + lS * grad[3];
      gcz = (double)(lS * grad[4]);
    }
    T lW0 = lw, lW1 = lhu, lW2 = lhv;
    T lb0 = 0, lb1 = 0, lb2 = 0;
    if (a.stage2) {  // out = 0.5*(Ubase + W): half to each
      lW0 = (T)0.5 * lw;
      lW1 = (T)0.5 * lhu;
      lW2 = (T)0.5 * lhv;
      a.lam_base[o] = lW0;
      a.lam_base[g.PS + o] = lW1;
      a.lam_base[2 * g.PS + o] = lW2;
    } else {  // stage 1: its input is U^n, which the stage-2 average saw too
      lb0 = a.lam_base[o];
      lb1 = a.lam_base[g.PS + o];
      lb2 = a.lam_base[2 * g.PS + o];
    }
    a.lamL[o] = tdt * lW0;
    a.lamL[g.PS + o] = tdt * lW1;
    a.lamL[2 * g.PS + o] = tdt * lW2;
    a.lam_direct[o] = (lq0 + lW0) + lb0;
    a.lam_direct[g.PS + o] = (lq1 + lW1) + lb1;
    a.lam_direct[2 * g.PS + o] = (lq2 + lW2) + lb2;
    a.gBc[o] = gbc;
  }
  red[tid] = gcz;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (tid < s) red[tid] += red[tid + s];
    __syncthreads();
  }
  if (tid == 0) a.gCz_part[blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// Reverse of minmod_slope (src/reconstruction/linearreconstruction.jl:28-43):
// adds d(slope)/d(l, c, r) * ls to (ll, lc, lr), following the operand the
// forward minmod returned.
template <typename T>
__device__ __forceinline__ void minmod_slope_rev(T l, T c, T r, T theta, T ls, T& ll, T& lc, T& lr) {
  using A = Arith<T>;
  const T fwd = r - c, bwd = c - l;
  const T ma = theta * fwd, mb = (fwd + bwd) * (T)0.5, mc = theta * bwd;
  int pick = -1;
  if (A::gt0(ma) && A::gt0(mb) && A::gt0(mc)) {
    const T m1 = A::min(ma, mb);
    const int p1 = (m1 == ma && !Arith<Dual<T>>::picks_second_min(ma, mb)) ? 0 : 1;
    const T m2 = A::min(m1, mc);
    pick = (m2 == m1 && !Arith<Dual<T>>::picks_second_min(m1, mc)) ? p1 : 2;
  } else if (A::lt0(ma) && A::lt0(mb) && A::lt0(mc)) {
    const T m1 = A::max(ma, mb);
    const int p1 = (m1 == ma && !Arith<Dual<T>>::picks_second_max(ma, mb)) ? 0 : 1;
    const T m2 = A::max(m1, mc);
    pick = (m2 == m1 && !Arith<Dual<T>>::picks_second_max(m1, mc)) ? p1 : 2;
  }
  T lf = 0, lb = 0;
  if (pick == 0) lf = theta * ls;
  if (pick == 1) {
    lf = (T)0.5 * ls;
    lb = (T)0.5 * ls;
  }
  if (pick == 2) lb = theta * ls;
  lr = lr + lf;
  lc = lc - lf + lb;
  ll = ll - lb;
}

// Per cell of the reconstruction range along DIR (the first ghost layer
// included, src/reconstruction/linearreconstruction.jl:60-68), interior across.
template <typename T, int DIR>
__global__ void __launch_bounds__(128) k_adj_recon(AdjArgs<T> a) {
  using A = Arith<T>;
  const Geom<T>& g = a.g;
  const Phys<T>& p = a.p;
  // along: cells gc-1 .. gc+n; across: interior
  const int n_al = DIR == 0 ? g.nx : g.ny;
  const int n_ac = DIR == 0 ? g.ny : g.nx;
  const int al = g.gc - 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int ac = g.gc + blockIdx.y * blockDim.y + threadIdx.y;
  if (al > g.gc + n_al || ac >= g.gc + n_ac) return;
  auto X = [&](int s) { return DIR == 0 ? al + s : ac; };
  auto Y = [&](int s) { return DIR == 0 ? ac : al + s; };
  auto ld = [&](int s, int k) -> T {
    const int xx = X(s), yy = Y(s);
    if (xx < 0 || yy < 0 || xx >= g.N1 || yy >= g.N2) return (T)0;
    return a.Uprev[k * g.PS + sidx(g, xx, yy)];
  };
  auto lamL = [&](int s, int k) -> T {  // lambda of L at an interior cell, else 0
    const int at = al + s;
    if (at < g.gc || at >= g.gc + n_al) return (T)0;
    return a.lamL[k * g.PS + sidx(g, X(s), Y(s))];
  };
  // bottom faces of cell at offset s along DIR
  auto bface = [&](int s, int right) -> T {
    if (g.bottom_const) return g.bconst;
    const int xx = X(s), yy = Y(s);
    const long long b = (long long)yy * g.PB + xx + XOFF;
    if (DIR == 0) {
      return right ? (T)0.5 * (a.B[b + 1] + a.B[b + 1 + g.PB]) : (T)0.5 * (a.B[b] + a.B[b + g.PB]);
    }
    return right ? (T)0.5 * (a.B[b + g.PB] + a.B[b + g.PB + 1]) : (T)0.5 * (a.B[b] + a.B[b + 1]);
  };
  // B_cell of the cell at offset s along DIR, in the forward kernels' order
  // (NoReconstruction's face depth is w - B_cell, src/reconstruction/noreconstruction.jl:30-46)
  auto bcell = [&](int s) -> T {
    if (g.bottom_const) return g.bconst;
    const long long b = (long long)Y(s) * g.PB + X(s) + XOFF;
    return (T)0.25 * (((a.B[b] + a.B[b + 1]) + a.B[b + g.PB]) + a.B[b + g.PB + 1]);
  };
  const T inv = DIR == 0 ? p.inv_dx : p.inv_dy;
  // Stencil values at offsets -2..+2 (only what is used is read).
  T u[5][3];
#pragma unroll
  for (int s = 0; s < 5; ++s)
#pragma unroll
    for (int k = 0; k < 3; ++k) u[s][k] = ld(s - 2, k);
  const bool face_r = al <= g.gc + n_al - 1;  // face c+1/2 is used
  const bool face_l = al >= g.gc;             // face c-1/2 is used
  // reconstruction of cells c-1, c, c+1 (forward)
  T Lc[3], Rc[3], Rm[3], Lp[3];
  const T Blc = bface(0, 0), Brc = bface(0, 1);
  if (p.rec_none) {
    no_reconstruction<T>(u[2], bcell(0), Lc, Rc);
    T tmp[3];
    if (face_l) no_reconstruction<T>(u[1], bcell(-1), tmp, Rm);
    if (face_r) no_reconstruction<T>(u[3], bcell(1), Lp, tmp);
  } else {
    reconstruct_cell<T>(p, u[1], u[2], u[3], Blc, Brc, Lc, Rc);
    if (face_l) {
      T Lm[3];
      reconstruct_cell<T>(p, u[0], u[1], u[2], bface(-1, 0), bface(-1, 1), Lm, Rm);
    }
    if (face_r) {
      T Rp[3];
      reconstruct_cell<T>(p, u[2], u[3], u[4], bface(1, 0), bface(1, 1), Lp, Rp);
    }
  }
  T lR[3] = {0, 0, 0}, lL[3] = {0, 0, 0};
  const Phys<Dual<T>> dp = dual_phys(p);
  if (face_r) {  // face between c and c+1: c is the minus side
    T lF[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) lF[k] = inv * (lamL(1, k) - lamL(0, k));
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      Dual<T> m[3], q[3], F[3], sp;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        m[k] = Dual<T>(Rc[k], j == k ? (T)1 : (T)0);
        q[k] = Dual<T>(Lp[k], (T)0);
      }
      cu_face<Dual<T>, DIR, false>(dp, m[0], m[1], m[2], q[0], q[1], q[2], F[0], F[1], F[2], sp);
      lR[j] = (lF[0] * F[0].d + lF[1] * F[1].d) + lF[2] * F[2].d;
    }
  }
  if (face_l) {  // face between c-1 and c: c is the plus side
    T lF[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) lF[k] = inv * (lamL(0, k) - lamL(-1, k));
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      Dual<T> m[3], q[3], F[3], sp;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        m[k] = Dual<T>(Rm[k], (T)0);
        q[k] = Dual<T>(Lc[k], j == k ? (T)1 : (T)0);
      }
      cu_face<Dual<T>, DIR, false>(dp, m[0], m[1], m[2], q[0], q[1], q[2], F[0], F[1], F[2], sp);
      lL[j] = (lF[0] * F[0].d + lF[1] * F[1].d) + lF[2] * F[2].d;
    }
  }
  // bottom source of interior cells (src/sourceterms/source_term_bottom.jl:24-41)
  T gBl = 0, gBr = 0;
  if (face_l && face_r && p.n_bottom > 0) {
    const int kk = DIR == 0 ? 1 : 2;
    const T lk = lamL(0, kk) * (T)p.n_bottom;
    const T slope = slope_over<T>(Brc - Blc, DIR == 0 ? p.dx : p.dy, inv, DIR == 0 ? p.dx_pow2 : p.dy_pow2);
    const T hmean = (Rc[0] + Lc[0]) * (T)0.5;
    lR[0] = lR[0] + lk * p.neg_g * slope * (T)0.5;
    lL[0] = lL[0] + lk * p.neg_g * slope * (T)0.5;
    const T ldb = lk * p.neg_g * hmean * inv;  // d(dB/Δ)/d(dB) = 1/Δ
    gBr = gBr + ldb;
    gBl = gBl - ldb;
  }
  // reconstruction of cell c in reverse
  T lu[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // [neighbour -1, 0, +1][component]
  if (p.rec_none) {
    // L = R = (w - B_cell, hu, hv): the cell takes both faces' lambda, and
    // d/dB_cell = -(lambda_L.h + lambda_R.h) goes to the corners a quarter
    // each, i.e. half to each face bottom of this direction (whose corners
    // are the cell's, a half each)
#pragma unroll
    for (int k = 0; k < 3; ++k) lu[1][k] = lL[k] + lR[k];
    const T dBc = (T)0 - (lL[0] + lR[0]);
    gBl = gBl + (T)0.5 * dBc;
    gBr = gBr + (T)0.5 * dBc;
  }
#pragma unroll
  for (int k = 1; k < 3 && !p.rec_none; ++k) {  // hu, hv: L = c - s/2, R = c + s/2
    lu[1][k] = lu[1][k] + lL[k] + lR[k];
    const T ls = (T)0.5 * (lR[k] - lL[k]);
    minmod_slope_rev<T>(u[1][k], u[2][k], u[3][k], p.theta, ls, lu[0][k], lu[1][k], lu[2][k]);
  }
  if (!p.rec_none) {  // w with the bottom-limited slope
    const T w = u[2][0];
    const T s0 = minmod_slope<T>(u[1][0], u[2][0], u[3][0], p.theta);
    // L0 = (w - s/2) - Bl, R0 = (w + s/2) - Br
    lu[1][0] = lu[1][0] + lL[0] + lR[0];
    gBl = gBl - lL[0];
    gBr = gBr - lR[0];
    const T ls = (T)0.5 * (lR[0] - lL[0]);
    if (A::lt(w - (T)0.5 * s0, Blc)) {          // s = 2(w - Bl)
      lu[1][0] = lu[1][0] + (T)2 * ls;
      gBl = gBl - (T)2 * ls;
    } else if (A::lt(w + (T)0.5 * s0, Brc)) {   // s = 2(Br - w)
      lu[1][0] = lu[1][0] - (T)2 * ls;
      gBr = gBr + (T)2 * ls;
    } else {
      minmod_slope_rev<T>(u[1][0], u[2][0], u[3][0], p.theta, ls, lu[0][0], lu[1][0], lu[2][0]);
    }
  }
  const long long o = sidx(g, X(0), Y(0));
  T* C = a.C[DIR];
#pragma unroll
  for (int nb = 0; nb < 3; ++nb)
#pragma unroll
    for (int k = 0; k < 3; ++k) C[(nb * 3 + k) * g.PS + o] = lu[nb][k];
  a.gBf[DIR][o] = gBl;
  a.gBf[DIR][g.PS + o] = gBr;
}

// lambda of the stage input per interior cell: direct part + neighbour
// contributions, with the lambda of wall ghost cells folded onto the interior
// cells they mirror (src/bc.jl:81-110; x ghosts negate hu, y ghosts hv).
template <typename T>
__global__ void __launch_bounds__(256) k_adj_gather(AdjArgs<T> a) {
  const Geom<T>& g = a.g;
  const int x = g.gc + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = g.gc + blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= g.gc + g.nx || y >= g.gc + g.ny) return;
  // contributions landing on cell (xx, yy) from the reconstructions along DIR
  auto land = [&](int dir, int xx, int yy, int k) -> T {
    const int al = dir == 0 ? xx : yy;
    const int n = dir == 0 ? g.nx : g.ny;
    const T* C = a.C[dir];
    T s = 0;
    // from the cell itself (to c), from c-1 (to c+1), from c+1 (to c-1)
    auto in_range = [&](int c) { return c >= g.gc - 1 && c <= g.gc + n; };
    if (in_range(al)) s = s + C[(3 + k) * g.PS + sidx(g, xx, yy)];
    if (in_range(al - 1)) {
      const int px = dir == 0 ? xx - 1 : xx, py = dir == 0 ? yy : yy - 1;
      s = s + C[(6 + k) * g.PS + sidx(g, px, py)];
    }
    if (in_range(al + 1)) {
      const int px = dir == 0 ? xx + 1 : xx, py = dir == 0 ? yy : yy + 1;
      s = s + C[(0 + k) * g.PS + sidx(g, px, py)];
    }
    return s;
  };
  const long long o = sidx(g, x, y);
  T lam[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) lam[k] = a.lam_direct[k * g.PS + o] + land(0, x, y, k) + land(1, x, y, k);
  // ghosts copying this cell: wall ghosts mirror it, x' = 2gc-1-x (left) or
  // 2(gc+nx)-1-x (right), with the normal momentum negated; periodic ghosts
  // repeat it a period away, x' = x + n (right) or x - n (left)
  // (src/bc.jl:29-40, 81-110)
#pragma unroll
  for (int dir = 0; dir < 2; ++dir) {
    const int v = dir == 0 ? x : y;
    const int n = dir == 0 ? g.nx : g.ny;
    int gh[2] = {-1, -1};
    if (g.bc == 2) {
      if (v - n >= 0 && v - n < g.gc) gh[0] = v - n;            // left/bottom ghost
      if (v + n >= g.gc + n && v + n < 2 * g.gc + n) gh[1] = v + n;  // right/top ghost
    } else {
      if (v < 2 * g.gc) gh[0] = 2 * g.gc - 1 - v;                  // left/bottom ghost
      if (v >= g.gc + n - g.gc) gh[1] = 2 * (g.gc + n) - 1 - v;    // right/top ghost
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int q = gh[s];
      if (q < 0 || (q >= g.gc && q < g.gc + n)) continue;
      const int gx = dir == 0 ? q : x, gy = dir == 0 ? y : q;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const T l = land(dir, gx, gy, k);
        const bool normal = g.bc == 1 && ((dir == 0 && k == 1) || (dir == 1 && k == 2));
        lam[k] = lam[k] + (normal ? -l : l);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) a.lam_in[k * g.PS + o] = lam[k];
}

// dLoss/dB per corner (I, J) of the (N1+1) x (N2+1) corner grid.
template <typename T>
__global__ void __launch_bounds__(256) k_adj_corner(AdjArgs<T> a) {
  const Geom<T>& g = a.g;
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  if (I > g.N1 || J > g.N2) return;
  auto cellv = [&](const T* arr, int cx, int cy) -> double {
    if (cx < 0 || cy < 0 || cx >= g.N1 || cy >= g.N2) return 0.0;
    return (double)arr[sidx(g, cx, cy)];
  };
  auto interior = [&](int cx, int cy) {
    return cx >= g.gc && cx < g.gc + g.nx && cy >= g.gc && cy < g.gc + g.ny;
  };
  double s = 0.0;
  // B_cell of the four cells sharing the corner
  double sc = 0.0;
  for (int dy = -1; dy <= 0; ++dy)
    for (int dx = -1; dx <= 0; ++dx)
      if (interior(I + dx, J + dy)) sc += cellv(a.gBc, I + dx, J + dy);
  s += 0.25 * sc;
  // face bottoms: x faces (left of cell (I, J) and (I, J-1); right of (I-1, J), (I-1, J-1))
  const T* fx = a.gBf[0];
  const T* fy = a.gBf[1];
  double sf = 0.0;
  sf += cellv(fx, I, J) + cellv(fx, I, J - 1);
  sf += cellv(fx + g.PS, I - 1, J) + cellv(fx + g.PS, I - 1, J - 1);
  // y faces (bottom of (I, J), (I-1, J); top of (I, J-1), (I-1, J-1))
  sf += cellv(fy, I, J) + cellv(fy, I - 1, J);
  sf += cellv(fy + g.PS, I, J - 1) + cellv(fy + g.PS, I - 1, J - 1);
  s += 0.5 * sf;
  a.gB[(long long)J * (g.N1 + 1) + I] += s;
}

// lambda of the final state from the gauge loss sum_g (w[g] - target[g])^2,
// and the loss, in gauge order (one thread).
template <typename T>
__global__ void k_adj_seed(Geom<T> g, const T* U, T* lam, const int* gi, const int* gj, const double* target, int n,
                           double* loss) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double L = 0.0;
  for (int k = 0; k < n; ++k) {
    const long long o = sidx(g, g.gc + gi[k], g.gc + gj[k]);
    const double d = (double)U[o] - target[k];
    L += d * d;
    lam[o] = (T)((double)lam[o] + 2.0 * d);
  }
  *loss = L;
}

// Sum of the per-block dLoss/dCz partials into *acc, in block order (one thread).
static __global__ void k_adj_sum(const double* part, int n, double* acc) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += part[i];
  *acc += s;
}

}  // namespace vf
