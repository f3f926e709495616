// vf_march.cuh -- column-marching step kernels.
//
// Each warp owns a strip of 32 consecutive columns: lanes 2..29 produce the 28
// output columns, lanes 0-1 and 30-31 are the 2-cell halo. The warp marches up
// a segment of SEG rows keeping a 3-row register window of (w, hu, hv); the
// y-direction reconstruction, central-upwind face flux and bottom source are
// carried from row to row in registers, and x-neighbours come from warp
// shuffles. No shared memory and no block-wide barrier: every face flux of the
// strip is computed once (plus the halo faces), which is what matters on
// GB300 where the Float64 pipe is 1/64 of the Float32 rate and Float32 is
// instruction-issue bound.
//
// flux pass  (k_flux_march):  L(U0) of src/system.jl:62-75, S(U0) of
//            src/friction.jl:62-78, CFL maxima (src/numericalflux/numericalflux.jl:32).
// stage pass (k_stage_march): U1 = clamp((U0 + dt*L) ./ (1 .- dt*[0,S,S])) with its
//            wall ghosts, formed on the fly for every loaded row; then stage 2 on U1,
//            the RK2 average, friction, dry clamp and U2's wall ghosts
//            (src/timestepper/rungekutta.jl:26-52, src/simulator.jl:145-177).
#pragma once
#include <type_traits>
#include "vf_kernels.cuh"

namespace vf {

constexpr int MW = 32;        // lanes per strip
constexpr int MOUT = 28;      // output columns per strip
constexpr int MWPB = 4;       // warps (strips) per block
// Desingularisation without a branch (desing<T, true>) in the Float32 flux
// pass, with the branch in the stage pass: at 4096^2 the flux pass measured
// 0.334 instead of 0.343 ms with it; the stage pass, held to 64 registers,
// spills more with it and measured 0.485 instead of 0.475 ms. Same bits.
constexpr bool kFluxSel = true;
constexpr bool kStageSel = false;

template <typename T>
__device__ __forceinline__ T shfl_up1(T v) { return __shfl_up_sync(0xffffffffu, v, 1); }
template <typename T>
__device__ __forceinline__ T shfl_dn1(T v) { return __shfl_down_sync(0xffffffffu, v, 1); }
template <typename T>
__device__ __forceinline__ T shfl_idx(T v, int src) { return __shfl_sync(0xffffffffu, v, src); }

struct StripGeom {
  int lane, x, xs;     // lane, its column, first output column
  int ys, ye;          // output rows [ys, ye)
  bool out_col;        // lane holds an output column inside the domain
  bool ld_col;         // column inside the stored array
  bool xedge;          // some lane of the strip is a ghost column or one of the two columns next to one
};

// Strip `strip`, row segment `seg` (of seg_rows rows) for the calling warp.
template <typename T>
__device__ __forceinline__ bool strip_setup_at(const Geom<T>& g, int seg_rows, int strip, int seg, StripGeom& s) {
  s.lane = threadIdx.x & (MW - 1);
  const int nstrips = (g.nx + MOUT - 1) / MOUT;
  if (strip >= nstrips) return false;
  s.xs = g.gc + strip * MOUT;
  s.x = s.xs - 2 + s.lane;
  s.ys = g.gc + seg * seg_rows;
  s.ye = min(s.ys + seg_rows, g.gc + g.ny);
  s.out_col = s.lane >= 2 && s.lane < 2 + MOUT && s.x < g.gc + g.nx;
  s.ld_col = s.x < g.N1;
  // Lanes span columns xs-2 .. xs+29; ghost columns are < gc and >= gc+nx,
  // and the two interior columns beside each side write wall ghosts.
  s.xedge = s.xs - 2 <= g.gc + 1 || s.xs + (MW - 3) >= g.gc + g.nx - 2;
  return true;
}

template <typename T>
__device__ __forceinline__ bool strip_setup(const Geom<T>& g, int seg_rows, StripGeom& s) {
  return strip_setup_at(g, seg_rows, (int)(blockIdx.x * MWPB + (threadIdx.x >> 5)), (int)blockIdx.y, s);
}

// Bottom corners (x, r) and (x+1, r) of one corner row.
template <typename T>
struct CornerRow {
  T a, b;
};

template <typename T>
__device__ __forceinline__ CornerRow<T> load_corner_row(const Geom<T>& g, const T* __restrict__ B, int x, int r) {
  CornerRow<T> c{g.bconst, g.bconst};
  if (!g.bottom_const) {
    c.a = c.b = (T)0;
    if (r <= g.N2) {
      const long long o = (long long)r * g.PB + x + XOFF;
      if (x <= g.N1) c.a = B[o];
      if (x + 1 <= g.N1) c.b = B[o + 1];
    }
  }
  return c;
}

// Lookups of src/bottom_topography.jl:97-101 from two corner rows (lo = row of
// the cell, hi = the row above).
template <typename T>
__device__ __forceinline__ T b_cell(const Geom<T>& g, const CornerRow<T>& lo, const CornerRow<T>& hi) {
  if (g.bottom_const) return g.bconst;
  return (T)0.25 * (((lo.a + lo.b) + hi.a) + hi.b);
}
template <typename T>
__device__ __forceinline__ T b_xface_l(const Geom<T>& g, const CornerRow<T>& lo, const CornerRow<T>& hi) {
  if (g.bottom_const) return g.bconst;
  return (T)0.5 * (lo.a + hi.a);
}
template <typename T>
__device__ __forceinline__ T b_yface(const Geom<T>& g, const CornerRow<T>& r) {
  if (g.bottom_const) return g.bconst;
  return (T)0.5 * (r.a + r.b);
}

template <typename T>
struct Cell3 {
  T w, hu, hv;
};

template <typename T, bool CG>
__device__ __forceinline__ Cell3<T> load_cell(const Geom<T>& g, const T* U, int x, int r, bool ok) {
  Cell3<T> c{(T)0, (T)0, (T)0};
  if (ok && r < g.N2) {
    const long long o = sidx(g, x, r);
    c.w = gld<CG>(U + o);
    c.hu = gld<CG>(U + g.PS + o);
    c.hv = gld<CG>(U + 2 * g.PS + o);
  }
  return c;
}

// Reconstruction of this lane's cell along y (DIR 1) or x (DIR 0).
template <typename T>
__device__ __forceinline__ void recon(const Phys<T>& p, const Cell3<T>& l, const Cell3<T>& c, const Cell3<T>& r, T Bl,
                                      T Br, Cell3<T>& L, Cell3<T>& R) {
  const T lv[3] = {l.w, l.hu, l.hv}, cv[3] = {c.w, c.hu, c.hv}, rv[3] = {r.w, r.hu, r.hv};
  T Lv[3], Rv[3];
  reconstruct_cell<T>(p, lv, cv, rv, Bl, Br, Lv, Rv);
  L = Cell3<T>{Lv[0], Lv[1], Lv[2]};
  R = Cell3<T>{Rv[0], Rv[1], Rv[2]};
}

template <typename T, int DIR, bool SPEED, bool SEL>
__device__ __forceinline__ Cell3<T> face(const Phys<T>& p, const Cell3<T>& m, const Cell3<T>& q, T& speed) {
  Cell3<T> F;
  cu_face<T, DIR, SPEED, SEL>(p, m.w, m.hu, m.hv, q.w, q.hu, q.hv, F.w, F.hu, F.hv, speed);
  return F;
}

// Bottom source of one direction added to acc (src/sourceterms/source_term_bottom.jl:34-40):
// once per SourceTermBottom entry in order; Float32 adds n_bottom * (-g) times
// the term at once (no loop; the same value for the usual single entry up to
// where multiply-add contraction falls).
template <typename T>
__device__ __forceinline__ T add_bottom(const Phys<T>& p, T acc, T slope, T hmean) {
  if constexpr (sizeof(T) == 4) {
    return acc + p.bottom_g * slope * hmean;
  } else {
    for (int b = 0; b < p.n_bottom; ++b) acc = acc + p.neg_g * slope * hmean;
    return acc;
  }
}

// x-direction contribution of row j for this lane: -(1/Δx)(F_{x+1/2} - F_{x-1/2})
// plus the bottom source along x (src/numericalflux/numericalflux.jl:24-30,
// src/sourceterms/source_term_bottom.jl:34-40). Every lane participates in the
// shuffles; lanes 2..30 compute valid faces x-1/2.
template <typename T, bool SPEED, bool SEL>
__device__ __forceinline__ Cell3<T> x_derivative(const Geom<T>& g, const Phys<T>& p, const Cell3<T>& u,
                                                 const CornerRow<T>& clo, const CornerRow<T>& chi, T& sx) {
  Cell3<T> ul{shfl_up1(u.w), shfl_up1(u.hu), shfl_up1(u.hv)};
  Cell3<T> ur{shfl_dn1(u.w), shfl_dn1(u.hu), shfl_dn1(u.hv)};
  const T bl = b_xface_l(g, clo, chi);
  const T br = shfl_dn1(bl);  // right x-face of x == left x-face of x+1
  Cell3<T> L, R;
  recon<T>(p, ul, u, ur, bl, br, L, R);
  const Cell3<T> Rm{shfl_up1(R.w), shfl_up1(R.hu), shfl_up1(R.hv)};
  T sp = (T)0;
  const Cell3<T> Fl = face<T, 0, SPEED, SEL>(p, Rm, L, sp);  // face x-1/2
  if (SPEED) sx = sp;
  const Cell3<T> Fr{shfl_dn1(Fl.w), shfl_dn1(Fl.hu), shfl_dn1(Fl.hv)};
  Cell3<T> acc;
  acc.w = (T)0 - p.inv_dx * (Fr.w - Fl.w);
  acc.hu = (T)0 - p.inv_dx * (Fr.hu - Fl.hu);
  acc.hv = (T)0 - p.inv_dx * (Fr.hv - Fl.hv);
  acc.hu = add_bottom<T>(p, acc.hu, slope_over<T>(br - bl, p.dx, p.inv_dx, p.dx_pow2), (R.w + L.w) * (T)0.5);
  return acc;
}

// March state of the y direction: reconstruction of row j and flux of face j-1/2.
template <typename T>
struct YCarry {
  Cell3<T> R;     // right (upper) face value of row j
  T Lh;           // left (lower) face depth of row j
  T Bl, Br;       // y-face bottoms of row j
  Cell3<T> Gm;    // flux through face j-1/2
};

__device__ __forceinline__ void warp_speed_max(unsigned long long& k) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) k = max(k, __shfl_xor_sync(0xffffffffu, k, o));
}

// Block reduction of the per-warp CFL maxima, one atomicMax per direction.
__device__ __forceinline__ void block_speed_commit(StepRecord* rec, int parity, unsigned long long kx,
                                                   unsigned long long ky) {
  __shared__ unsigned long long red[2][MWPB];
  warp_speed_max(kx);
  warp_speed_max(ky);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = kx;
    red[1][threadIdx.x >> 5] = ky;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    unsigned long long m = 0;
#pragma unroll
    for (int w = 0; w < MWPB; ++w) m = max(m, red[threadIdx.x][w]);
    if (m) atomicMax(&rec->speed_bits[parity][threadIdx.x], m);
  }
}

// ---------------------------------------------------------------------------
// Flux pass of one strip segment (warp-collective): L(U0), S(U0); mx, my
// collect the warp's CFL maxima as bit-pattern keys.
template <typename T, bool CG>
__device__ __forceinline__ void flux_march_unit(const Geom<T>& g, const Phys<T>& p, const T* U,
                                                const T* __restrict__ B, T* Lout, T* Sout, const StripGeom& s,
                                                unsigned long long& mx_out, unsigned long long& my_out) {
  // Float32 speed keys fit 32 bits: one 32-bit max per face instead of a
  // 64-bit one (the flux pass measured 0.367 instead of 0.385 ms at 4096^2).
  using Key = typename std::conditional<sizeof(T) == 4, unsigned, unsigned long long>::type;
  Key mx = 0, my = 0;
  const int x = s.x;
  // prologue: rows ys-2..ys+1, corner rows ys-1..ys+2
  const Cell3<T> um2 = load_cell<T, CG>(g, U, x, s.ys - 2, s.ld_col);
  const Cell3<T> um1 = load_cell<T, CG>(g, U, x, s.ys - 1, s.ld_col);
  Cell3<T> uc = load_cell<T, CG>(g, U, x, s.ys, s.ld_col);
  Cell3<T> un = load_cell<T, CG>(g, U, x, s.ys + 1, s.ld_col);
  const CornerRow<T> cm1 = load_corner_row(g, B, x, s.ys - 1);
  CornerRow<T> c0 = load_corner_row(g, B, x, s.ys);
  CornerRow<T> c1 = load_corner_row(g, B, x, s.ys + 1);
  YCarry<T> y;
  {
    Cell3<T> Lm, Rm, L0, R0;
    const T blm = b_yface(g, cm1), b0 = b_yface(g, c0), b1 = b_yface(g, c1);
    recon<T>(p, um2, um1, uc, blm, b0, Lm, Rm);  // row ys-1
    recon<T>(p, um1, uc, un, b0, b1, L0, R0);    // row ys
    T sp = (T)0;
    y.Gm = face<T, 1, true, kFluxSel>(p, Rm, L0, sp);
    if (s.out_col) my = max(my, (Key)speed_key<T>(sp));
    y.R = R0;
    y.Lh = L0.w;
    y.Bl = b0;
    y.Br = b1;
  }
  for (int j = s.ys; j < s.ye; ++j) {
    const Cell3<T> u2 = load_cell<T, CG>(g, U, x, j + 2, s.ld_col);
    const CornerRow<T> c2 = load_corner_row(g, B, x, j + 2);
    T sx = (T)0;
    Cell3<T> acc = x_derivative<T, true, kFluxSel>(g, p, uc, c0, c1, sx);
    if (s.lane >= 2 && s.lane <= 2 + MOUT && s.x <= g.gc + g.nx) mx = max(mx, (Key)speed_key<T>(sx));
    // y: reconstruct row j+1, flux through face j+1/2
    Cell3<T> Ln, Rn;
    const T b2 = b_yface(g, c2);
    recon<T>(p, uc, un, u2, y.Br, b2, Ln, Rn);
    T sp = (T)0;
    const Cell3<T> Gp = face<T, 1, true, kFluxSel>(p, y.R, Ln, sp);
    if (s.out_col) my = max(my, (Key)speed_key<T>(sp));
    acc.w = acc.w - p.inv_dy * (Gp.w - y.Gm.w);
    acc.hu = acc.hu - p.inv_dy * (Gp.hu - y.Gm.hu);
    acc.hv = acc.hv - p.inv_dy * (Gp.hv - y.Gm.hv);
    acc.hv = add_bottom<T>(p, acc.hv, slope_over<T>(y.Br - y.Bl, p.dy, p.inv_dy, p.dy_pow2), (y.R.w + y.Lh) * (T)0.5);
    acc.w = add_point_sources<T>(p, acc.w);
    if (s.out_col) {
      const long long o = sidx(g, x, j);
      Lout[o] = acc.w;
      Lout[g.PS + o] = acc.hu;
      Lout[2 * g.PS + o] = acc.hv;
      if (p.friction) {
        T S = (T)0;
        if (friction_active<T>(uc.hu, uc.hv)) S = friction_factor<T>(p, uc.w, uc.hu, uc.hv, b_cell(g, c0, c1));
        Sout[o] = S;
      }
    }
    // shift the window
    uc = un;
    un = u2;
    c0 = c1;
    c1 = c2;
    y.R = Rn;
    y.Lh = Ln.w;
    y.Bl = y.Br;
    y.Br = b2;
    y.Gm = Gp;
  }
  mx_out = max(mx_out, (unsigned long long)mx);
  my_out = max(my_out, (unsigned long long)my);
}

// Resident blocks per SM the stage kernel is compiled for. The Float32 kernel
// otherwise takes 92 registers (five blocks, 20 warps) and waits on memory;
// at eight blocks (64 registers, a few bytes of spill) the 4096^2 stage pass
// measured 0.616 instead of 0.755 ms, and after the edge and source changes
// 0.475 against 0.551 ms at seven blocks (72 registers). The Float32 flux
// pass is held to seven blocks (72 registers, no spill): 0.319 instead of
// 0.323 ms at its natural 77 registers and six blocks. Float64 (190
// registers) is bound by the FP64 pipe and is left alone.
#ifndef VF_MARCH_STAGE_BLOCKS_F32
#define VF_MARCH_STAGE_BLOCKS_F32 8
#endif
#ifndef VF_MARCH_FLUX_BLOCKS_F32
#define VF_MARCH_FLUX_BLOCKS_F32 7
#endif
template <typename T> struct MarchStageBlocks { static constexpr int value = sizeof(T) == 4 ? VF_MARCH_STAGE_BLOCKS_F32 : 1; };
template <typename T> struct MarchFluxBlocks { static constexpr int value = sizeof(T) == 4 ? VF_MARCH_FLUX_BLOCKS_F32 : 1; };

template <typename T, int SEG>
__global__ void __launch_bounds__(MW * MWPB, MarchFluxBlocks<T>::value) k_flux_march(Geom<T> g, Phys<T> p, const T* __restrict__ U,
                                                          const T* __restrict__ B, T* __restrict__ Lout,
                                                          T* __restrict__ Sout, StepRecord* rec, int parity) {
  if (!rec->active[parity]) return;
  StripGeom s;
  unsigned long long mx = 0ull, my = 0ull;  // CFL maxima as bit patterns (speeds are >= 0)
  if (strip_setup(g, SEG, s)) flux_march_unit<T, false>(g, p, U, B, Lout, Sout, s, mx, my);
  block_speed_commit(rec, parity, mx, my);
}

// U1 of one loaded row for this lane (stage-1 update + dry clamp), before ghost mirroring.
template <typename T, bool CG>
__device__ __forceinline__ Cell3<T> stage1_row(const Geom<T>& g, const Phys<T>& p, T tdt, const T* U0, const T* Lin,
                                               const T* Sin, int x, int r, bool xin, const CornerRow<T>& clo,
                                               const CornerRow<T>& chi, Cell3<T>& u0out) {
  Cell3<T> u1{(T)0, (T)0, (T)0};
  u0out = Cell3<T>{(T)0, (T)0, (T)0};
  const bool yin = r >= g.gc && r < g.gc + g.ny;
  if (xin && yin) {
    const long long o = sidx(g, x, r);
    u0out = Cell3<T>{gld<CG>(U0 + o), gld<CG>(U0 + g.PS + o), gld<CG>(U0 + 2 * g.PS + o)};
    const T S = p.friction ? gld<CG>(Sin + o) : (T)0;
    stage1_point<T>(p, tdt, u0out.w, u0out.hu, u0out.hv, gld<CG>(Lin + o), gld<CG>(Lin + g.PS + o),
                    gld<CG>(Lin + 2 * g.PS + o), S, b_cell(g, clo, chi), u1.w, u1.hu, u1.hv);
  }
  return u1;
}

// Wall ghost columns of a U1 row (src/bc.jl:92-100): ghost lanes read their
// mirror source lane, hu negated. Every lane takes part in the shuffles.
template <typename T>
__device__ __forceinline__ Cell3<T> mirror_columns(const Geom<T>& g, const StripGeom& s, const Cell3<T>& u, bool yin) {
  if (!s.xedge) return u;  // warp-uniform: no ghost column in this strip
  int src = s.lane;
  bool ghost = false;
  if (yin && s.x < g.gc) {
    src = s.lane + (2 * g.gc - 1 - 2 * s.x);
    ghost = true;
  } else if (yin && s.x >= g.gc + g.nx && s.x < g.N1) {
    src = s.lane + (2 * (g.gc + g.nx) - 1 - 2 * s.x);
    ghost = true;
  }
  src = min(max(src, 0), MW - 1);
  Cell3<T> m{shfl_idx(u.w, src), shfl_idx(u.hu, src), shfl_idx(u.hv, src)};
  if (!ghost) return u;
  m.hu = -m.hu;
  return m;
}

template <typename T>
__device__ __forceinline__ Cell3<T> mirror_row(const Cell3<T>& src) {  // src/bc.jl:101-109, hv negated
  return Cell3<T>{src.w, src.hu, -src.hv};
}

// U2 of cell (x, j) and the wall ghosts it is the mirror source of
// (src/bc.jl:81-110): what store_with_ghosts writes for a wall boundary, with
// the ghost logic skipped in warp-uniform branches for strips without ghost
// columns and rows away from the bottom and top. With mirror_columns' early
// return for such strips, the Float32 stage pass at 4096^2 measured 0.503
// instead of 0.543 ms (the same bits).
template <typename T>
__device__ __forceinline__ void store_march(const Geom<T>& g, const StripGeom& s, T* __restrict__ Uo, int x, int j, T w,
                                            T hu, T hv) {
  if (s.xedge || j < g.gc + 2 || j >= g.gc + g.ny - 2) {
    store_with_ghosts<T>(g, Uo, x, j, w, hu, hv);
    return;
  }
  const long long o = sidx(g, x, j);
  Uo[o] = w;
  Uo[g.PS + o] = hu;
  Uo[2 * g.PS + o] = hv;
}

// RK2 stage pass of one strip segment (warp-collective): U2 with its ghosts into Uo.
template <typename T, bool CG>
__device__ __forceinline__ void stage_march_unit(const Geom<T>& g, const Phys<T>& p, const T* U0,
                                                 const T* __restrict__ B, const T* Lin, const T* Sin, T* Uo,
                                                 const StripGeom& s, T tdt) {
  const int x = s.x;
  const bool xin = x >= g.gc && x < g.gc + g.nx;
  const int top = g.gc + g.ny;  // first top ghost row
  // prologue: corner rows ys-2..ys+2, U1 rows ys-2..ys+1
  const CornerRow<T> cm2 = load_corner_row(g, B, x, s.ys - 2);
  const CornerRow<T> cm1 = load_corner_row(g, B, x, s.ys - 1);
  CornerRow<T> c0 = load_corner_row(g, B, x, s.ys);
  CornerRow<T> c1 = load_corner_row(g, B, x, s.ys + 1);
  CornerRow<T> c2 = load_corner_row(g, B, x, s.ys + 2);
  Cell3<T> u0c{(T)0, (T)0, (T)0}, u0n{(T)0, (T)0, (T)0}, dummy;
  Cell3<T> uc = mirror_columns(g, s, stage1_row<T, CG>(g, p, tdt, U0, Lin, Sin, x, s.ys, xin, c0, c1, u0c), true);
  Cell3<T> un;
  if (s.ys + 1 >= top) {
    un = mirror_row(uc);  // top ghost above a one-row segment
  } else {
    un = mirror_columns(g, s, stage1_row<T, CG>(g, p, tdt, U0, Lin, Sin, x, s.ys + 1, xin, c1, c2, u0n), true);
  }
  Cell3<T> um1, um2;
  if (s.ys == g.gc) {  // bottom ghosts mirror rows gc, gc+1
    um1 = mirror_row(uc);
    um2 = mirror_row(un);
  } else {
    um1 = mirror_columns(g, s, stage1_row<T, CG>(g, p, tdt, U0, Lin, Sin, x, s.ys - 1, xin, cm1, c0, dummy), true);
    um2 = mirror_columns(g, s, stage1_row<T, CG>(g, p, tdt, U0, Lin, Sin, x, s.ys - 2, xin, cm2, cm1, dummy), true);
  }
  // Ghost row top+1 mirrors row top-2, which leaves the window before it is needed.
  Cell3<T> stash{(T)0, (T)0, (T)0};
  if (s.ys + 1 == top) stash = mirror_row(um1);
  YCarry<T> y;
  {
    Cell3<T> Lm, Rm, L0, R0;
    const T blm = b_yface(g, cm1), b0 = b_yface(g, c0), b1 = b_yface(g, c1);
    recon<T>(p, um2, um1, uc, blm, b0, Lm, Rm);
    recon<T>(p, um1, uc, un, b0, b1, L0, R0);
    T sp;
    y.Gm = face<T, 1, false, kStageSel>(p, Rm, L0, sp);
    y.R = R0;
    y.Lh = L0.w;
    y.Bl = b0;
    y.Br = b1;
  }
  for (int j = s.ys; j < s.ye; ++j) {
    // U1 of row j+2 (needs corner rows j+2, j+3)
    const CornerRow<T> c3 = load_corner_row(g, B, x, j + 3);
    Cell3<T> u2, u0x{(T)0, (T)0, (T)0};
    if (j + 2 == top) {
      u2 = mirror_row(un);     // row top mirrors top-1
      stash = mirror_row(uc);  // row top+1 mirrors top-2
    } else if (j + 2 == top + 1) {
      u2 = stash;
    } else {
      u2 = mirror_columns(g, s, stage1_row<T, CG>(g, p, tdt, U0, Lin, Sin, x, j + 2, xin, c2, c3, u0x), j + 2 < top);
    }
    T sx;
    Cell3<T> acc = x_derivative<T, false, kStageSel>(g, p, uc, c0, c1, sx);
    Cell3<T> Ln, Rn;
    const T b2 = b_yface(g, c2);
    recon<T>(p, uc, un, u2, y.Br, b2, Ln, Rn);
    T sp;
    const Cell3<T> Gp = face<T, 1, false, kStageSel>(p, y.R, Ln, sp);
    acc.w = acc.w - p.inv_dy * (Gp.w - y.Gm.w);
    acc.hu = acc.hu - p.inv_dy * (Gp.hu - y.Gm.hu);
    acc.hv = acc.hv - p.inv_dy * (Gp.hv - y.Gm.hv);
    acc.hv = add_bottom<T>(p, acc.hv, slope_over<T>(y.Br - y.Bl, p.dy, p.inv_dy, p.dy_pow2), (y.R.w + y.Lh) * (T)0.5);
    acc.w = add_point_sources<T>(p, acc.w);
    if (s.out_col) {
      T w = uc.w + tdt * acc.w;
      T hu = uc.hu + tdt * acc.hu;
      T hv = uc.hv + tdt * acc.hv;
      w = (T)0.5 * (u0c.w + w);
      hu = (T)0.5 * (u0c.hu + hu);
      hv = (T)0.5 * (u0c.hv + hv);
      const T Bc = b_cell(g, c0, c1);
      if (p.friction && friction_active<T>(uc.hu, uc.hv))
        apply_friction<T>(tdt, friction_factor<T>(p, uc.w, uc.hu, uc.hv, Bc), hu, hv);
      dry_clamp<T>(p, w, hu, hv, Bc);
      store_march<T>(g, s, Uo, x, j, w, hu, hv);
    }
    uc = un;
    un = u2;
    u0c = u0n;
    u0n = u0x;
    c0 = c1;
    c1 = c2;
    c2 = c3;
    y.R = Rn;
    y.Lh = Ln.w;
    y.Bl = y.Br;
    y.Br = b2;
    y.Gm = Gp;
  }
}

template <typename T, int SEG>
__global__ void __launch_bounds__(MW * MWPB, MarchStageBlocks<T>::value) k_stage_march(Geom<T> g, Phys<T> p, const T* __restrict__ U0,
                                                           const T* __restrict__ B, const T* __restrict__ Lin,
                                                           const T* __restrict__ Sin, T* __restrict__ Uo,
                                                           StepRecord* rec, int parity) {
  const bool root = blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0;
  if (!rec->active[parity]) {
    if (root) carry_record(rec, parity);
    return;
  }
  __shared__ double s_dt;
  if (threadIdx.x == 0) s_dt = step_dt<T>(g, rec, parity);
  __syncthreads();
  const double dt = s_dt;
  StripGeom s;
  if (strip_setup(g, SEG, s)) stage_march_unit<T, false>(g, p, U0, B, Lin, Sin, Uo, s, (T)dt);
  if (root) advance_record<T>(rec, parity, dt);
}

}  // namespace vf
