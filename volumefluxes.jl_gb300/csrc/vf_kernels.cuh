// vf_kernels.cuh -- the fused tile kernels of one RK2 / forward-Euler step.
//
// A step is two launches (three for nothing else):
//   flux pass   reads U0 (+2-cell halo) and B, computes the time derivative
//               L(U0) of src/system.jl:62-75 (x then y: reconstruction, central-
//               upwind fluxes, bottom source; then rain/infiltration), the
//               friction factor S(U0) of src/friction.jl:62-78, and the CFL
//               maxima (warp shuffles + one atomicMax per block per direction).
//   stage pass  (RK2) reads U0, L, S on the tile + halo, forms the stage-1
//               result U1 = clamp((U0 + dt*L) ./ (1 .- dt*[0,S,S])) pointwise in
//               shared memory with its wall ghosts, runs the whole stage-2
//               derivative on U1, then the Euler update, RK2 average, friction,
//               dry clamp and wall ghosts of U2 (src/timestepper/rungekutta.jl:26-52,
//               src/simulator.jl:145-177). dt comes from the flux pass's maxima
//               (src/simulator.jl:147-150) and is computed on the device.
//   apply pass  (forward Euler) the pointwise stage-1 update alone.
//
// Tiles are TX x TY interior cells; each block stages its tile with a 2-cell
// halo of (w, hu, hv) and a 2..3-cell halo of bottom corners in shared memory.
// The Float64 kernels of the per-step path (k_flux_tma, k_stage2_tma) stage
// them with TMA copies, and the stage pass writes its output tile with a TMA
// tensor store (vf_tma.cuh); the ensemble and Float32 tiles load and store
// the plain way.
#pragma once
#include "vf_math.cuh"
#include "vf_tma.cuh"

namespace vf {

constexpr int TX = 32;
constexpr int TY = 16;
constexpr int NT = 256;
constexpr int CPT = TX * TY / NT;  // cells per thread
constexpr int HX = TX + 4;
constexpr int HY = TY + 4;
constexpr int BHX = TX + 6;  // TX + 5 corner columns are read; one more keeps Float64 rows 16-byte multiples
constexpr int BHY = TY + 5;
constexpr int LRN = (TX + 2) * TY > TX * (TY + 2) ? (TX + 2) * TY : TX * (TY + 2);
constexpr int FN = (TX + 1) * TY > TX * (TY + 1) ? (TX + 1) * TY : TX * (TY + 1);
constexpr int XOFF = 2;  // leading pad columns in device rows
#ifndef VF_TILE_MIN_BLOCKS
#define VF_TILE_MIN_BLOCKS 1
#endif

// Device-resident step record. Slots indexed by step parity let every kernel
// of step n read slot n&1 while the stage pass prepares slot (n+1)&1.
struct StepRecord {
  unsigned long long speed_bits[2][2];  // CFL maxima (ax, ay) as IEEE bit patterns, >= 0
  double t[2];
  int active[2];
  int match_endtime;
  int has_max_ts;
  double endtime;
  double max_ts;
  double stop_time;
  double last_dt;
  long long n_done;
  double explicit_max_dt;
  int explicit_mode;
  int force_dt;        // 1: every step uses forced_dt (a frozen dt sequence)
  int wait_fault;      // set when a bounded wait for a tile copy gave up
  double forced_dt;
};

template <typename T>
struct Geom {
  int nx, ny, gc, N1, N2;
  long long P, PS, PB;  // state row pitch, plane stride, corner row pitch (elements)
  int bottom_const;
  T bconst;
  double dx, dy, cfl;
  int bc;  // 1 wall (src/bc.jl:81-110), 2 periodic (src/bc.jl:29-40)
};

// Interior source cell of ghost coordinate v (0 <= v < n + 2gc) along axis 0
// (x) or 1 (y): the mirror for walls (src/bc.jl:81-110), the opposite side for
// periodic boundaries (src/bc.jl:29-40). NeumannBC as src/bc.jl:49-60 writes
// it: the left columns mirror the interior, the bottom rows copy the top
// interior rows; its right and top ghosts have no source (neumann_outer).
__device__ __forceinline__ int bc_source(int v, int gc, int n, int bc, int axis) {
  if (bc == 2 || (bc == 3 && axis == 1 && v < gc)) return v < gc ? v + n : v - n;
  return v < gc ? 2 * gc - 1 - v : 2 * (gc + n) - 1 - v;
}

template <typename T>
__device__ __forceinline__ long long sidx(const Geom<T>& g, int x, int y) {
  return (long long)y * g.P + x + XOFF;
}

// Global load of step data. CG = true reads through L2 only (ld.global.cg): the
// ensemble kernel reads fields that other CTAs of its cluster wrote earlier in
// the same launch, which the read-only and L1 paths may not see.
template <bool CG, typename T>
__device__ __forceinline__ T gld(const T* ptr) {
  if constexpr (CG) {
    return __ldcg(ptr);
  } else {
    return *ptr;
  }
}

// Bottom topography seen from a tile; (lx, ly) are tile-local cell coordinates,
// corner (x0+lx, y0+ly) lives at sB[(ly+2)*BHX + lx+2]. Lookups follow
// src/bottom_topography.jl:97-101.
template <typename T>
struct BTile {
  const T* sB;
  int is_const;
  T c;
  __device__ __forceinline__ T cn(int lx, int ly) const { return sB[(ly + 2) * BHX + lx + 2]; }
  __device__ __forceinline__ T cell(int lx, int ly) const {
    if (is_const) return c;
    return (T)0.25 * (((cn(lx, ly) + cn(lx + 1, ly)) + cn(lx, ly + 1)) + cn(lx + 1, ly + 1));
  }
  template <int DIR>
  __device__ __forceinline__ T face_l(int lx, int ly) const {
    if (is_const) return c;
    return DIR == 0 ? (T)0.5 * (cn(lx, ly) + cn(lx, ly + 1)) : (T)0.5 * (cn(lx, ly) + cn(lx + 1, ly));
  }
  template <int DIR>
  __device__ __forceinline__ T face_r(int lx, int ly) const {
    if (is_const) return c;
    return DIR == 0 ? (T)0.5 * (cn(lx + 1, ly) + cn(lx + 1, ly + 1)) : (T)0.5 * (cn(lx, ly + 1) + cn(lx + 1, ly + 1));
  }
};

template <typename T>
__device__ __forceinline__ void load_corners(const Geom<T>& g, const T* __restrict__ B, T* sB, int x0, int y0) {
  for (int idx = threadIdx.x; idx < BHX * BHY; idx += NT) {
    const int bx = idx % BHX, by = idx / BHX;
    const int cx = x0 - 2 + bx, cy = y0 - 2 + by;
    T v = (T)0;
    if (cx <= g.N1 && cy <= g.N2) v = B[(long long)cy * g.PB + cx + XOFF];
    sB[idx] = v;
  }
}

// NoReconstruction for practical SWE, src/reconstruction/noreconstruction.jl:30-46:
// both face values are (w - B_cell, hu, hv).
template <typename T>
__device__ __forceinline__ void no_reconstruction(const T c[3], T Bc, T L[3], T R[3]) {
  L[0] = R[0] = c[0] - Bc;
  L[1] = R[1] = c[1];
  L[2] = R[2] = c[2];
}

// Stage-1 result U1 of one interior cell read straight from global memory
// (used for ghost cells, whose source may lie outside the tile).
template <typename T>
__device__ __forceinline__ void stage1_point(const Phys<T>& p, T tdt, T u0, T u1, T u2, T l0, T l1, T l2, T S, T Bc,
                                             T& w, T& hu, T& hv);
template <typename T, bool CG>
__device__ __forceinline__ void u1_global(const Geom<T>& g, const Phys<T>& p, T tdt, const T* U0, const T* Lin,
                                          const T* Sin, const T* __restrict__ B, int x, int y, T& w, T& hu, T& hv) {
  const long long o = sidx(g, x, y);
  T Bc = g.bconst;
  if (!g.bottom_const) {
    const long long b = (long long)y * g.PB + x + XOFF;
    Bc = (T)0.25 * (((B[b] + B[b + 1]) + B[b + g.PB]) + B[b + g.PB + 1]);
  }
  const T S = p.friction ? gld<CG>(Sin + o) : (T)0;
  stage1_point<T>(p, tdt, gld<CG>(U0 + o), gld<CG>(U0 + g.PS + o), gld<CG>(U0 + 2 * g.PS + o), gld<CG>(Lin + o),
                  gld<CG>(Lin + g.PS + o), gld<CG>(Lin + 2 * g.PS + o), S, Bc, w, hu, hv);
}

// Time derivative of one stage on the tile held in sU (3 planes of HY x HX).
// acc[k][*] receives -(1/Δx)(F_r-F_l) [+ bottom x], then -(1/Δy)(G_r-G_l)
// [+ bottom y] for the cells this thread owns (cell tid + k*NT, x fastest).
// src/system.jl:64-70 (directions in order), numericalflux.jl:21-33,
// linearreconstruction.jl:58-102, source_term_bottom.jl:24-41.
template <typename T, bool SPEED>
__device__ __forceinline__ void tile_derivative(const Phys<T>& p, const T* sU, const BTile<T>& bt, T* sL, T* sR, T* sF,
                                                T (&acc)[CPT][3], T& mx, T& my, int nvx, int nvy) {
  const int tid = threadIdx.x;
  // ---- x: reconstruct cells lx in [-1, TX], ly in [0, TY)
  for (int idx = tid; idx < (TX + 2) * TY; idx += NT) {
    const int lx = idx % (TX + 2) - 1, ly = idx / (TX + 2);
    const int c = (ly + 2) * HX + lx + 2;
    T l[3], m[3], r[3], L[3], R[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      l[k] = sU[k * HX * HY + c - 1];
      m[k] = sU[k * HX * HY + c];
      r[k] = sU[k * HX * HY + c + 1];
    }
    if (p.rec_none) {
      no_reconstruction<T>(m, bt.cell(lx, ly), L, R);
    } else {
      reconstruct_cell<T>(p, l, m, r, bt.template face_l<0>(lx, ly), bt.template face_r<0>(lx, ly), L, R);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      sL[k * LRN + idx] = L[k];
      sR[k * LRN + idx] = R[k];
    }
  }
  __syncthreads();
  // ---- x: faces f in [0, TX] between cells f-1 and f
  for (int idx = tid; idx < (TX + 1) * TY; idx += NT) {
    const int f = idx % (TX + 1), ly = idx / (TX + 1);
    const int im = ly * (TX + 2) + f, ip = im + 1;
    T F0, F1, F2, sp = (T)0;
    cu_face<T, 0, SPEED>(p, sR[im], sR[LRN + im], sR[2 * LRN + im], sL[ip], sL[LRN + ip], sL[2 * LRN + ip], F0, F1, F2,
                         sp);
    sF[idx] = F0;
    sF[FN + idx] = F1;
    sF[2 * FN + idx] = F2;
    if (SPEED && ly < nvy && f <= nvx) mx = fmax(mx, sp);
  }
  __syncthreads();
  // ---- x: accumulate
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    const int c = tid + k * NT;
    const int lx = c % TX, ly = c / TX;
    const int fl = ly * (TX + 1) + lx;
#pragma unroll
    for (int j = 0; j < 3; ++j) acc[k][j] = (T)0 - p.inv_dx * (sF[j * FN + fl + 1] - sF[j * FN + fl]);
    const int rc = ly * (TX + 2) + lx + 1;
    for (int b = 0; b < p.n_bottom; ++b) {
      const T Bl = bt.template face_l<0>(lx, ly), Br = bt.template face_r<0>(lx, ly);
      acc[k][1] = acc[k][1] + p.neg_g * slope_over<T>(Br - Bl, p.dx, p.inv_dx, p.dx_pow2) * ((sR[rc] + sL[rc]) * (T)0.5);
    }
  }
  __syncthreads();
  // ---- y: reconstruct cells lx in [0, TX), ly in [-1, TY]
  for (int idx = tid; idx < TX * (TY + 2); idx += NT) {
    const int lx = idx % TX, ly = idx / TX - 1;
    const int c = (ly + 2) * HX + lx + 2;
    T l[3], m[3], r[3], L[3], R[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      l[k] = sU[k * HX * HY + c - HX];
      m[k] = sU[k * HX * HY + c];
      r[k] = sU[k * HX * HY + c + HX];
    }
    if (p.rec_none) {
      no_reconstruction<T>(m, bt.cell(lx, ly), L, R);
    } else {
      reconstruct_cell<T>(p, l, m, r, bt.template face_l<1>(lx, ly), bt.template face_r<1>(lx, ly), L, R);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      sL[k * LRN + idx] = L[k];
      sR[k * LRN + idx] = R[k];
    }
  }
  __syncthreads();
  // ---- y: faces f in [0, TY] between cells f-1 and f
  for (int idx = tid; idx < TX * (TY + 1); idx += NT) {
    const int lx = idx % TX, f = idx / TX;
    const int im = f * TX + lx, ip = im + TX;
    T F0, F1, F2, sp = (T)0;
    cu_face<T, 1, SPEED>(p, sR[im], sR[LRN + im], sR[2 * LRN + im], sL[ip], sL[LRN + ip], sL[2 * LRN + ip], F0, F1, F2,
                         sp);
    sF[idx] = F0;
    sF[FN + idx] = F1;
    sF[2 * FN + idx] = F2;
    if (SPEED && lx < nvx && f <= nvy) my = fmax(my, sp);
  }
  __syncthreads();
  // ---- y: accumulate
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    const int c = tid + k * NT;
    const int lx = c % TX, ly = c / TX;
    const int fl = ly * TX + lx;
#pragma unroll
    for (int j = 0; j < 3; ++j) acc[k][j] = acc[k][j] - p.inv_dy * (sF[j * FN + fl + TX] - sF[j * FN + fl]);
    const int rc = (ly + 1) * TX + lx;
    for (int b = 0; b < p.n_bottom; ++b) {
      const T Bl = bt.template face_l<1>(lx, ly), Br = bt.template face_r<1>(lx, ly);
      acc[k][2] = acc[k][2] + p.neg_g * slope_over<T>(Br - Bl, p.dy, p.inv_dy, p.dy_pow2) * ((sR[rc] + sL[rc]) * (T)0.5);
    }
  }
}

template <typename T>
__device__ __forceinline__ unsigned long long speed_key(T v);
template <>
__device__ __forceinline__ unsigned long long speed_key<double>(double v) {
  return (unsigned long long)__double_as_longlong(v);
}
template <>
__device__ __forceinline__ unsigned long long speed_key<float>(float v) {
  return (unsigned long long)(unsigned)__float_as_uint(v);
}
template <typename T>
__device__ __forceinline__ double speed_from_key(unsigned long long k);
template <>
__device__ __forceinline__ double speed_from_key<double>(unsigned long long k) {
  return __longlong_as_double((long long)k);
}
template <>
__device__ __forceinline__ double speed_from_key<float>(unsigned long long k) {
  return (double)__uint_as_float((unsigned)k);
}

// ---------------------------------------------------------------------------
// Flux pass: L(U0), S(U0) and the CFL maxima.
// U and B come first: for Float64 both start 128-byte aligned (TMA destinations).
template <typename T>
struct SmemFlux {
  T U[3 * HX * HY];
  T B[BHX * BHY];
  T L[3 * LRN];
  T R[3 * LRN];
  T F[3 * FN];
  unsigned long long red[2][NT / 32];
  T scal[8];
  unsigned long long bar;  // mbarrier of the tile copies
  int plain;               // 0: staged by TMA; 1: not staged (alignment); 2: the wait gave up
};

// Flux pass over one tile at (x0, y0) (block-collective): L(U0) and S(U0) to
// global memory; mx, my accumulate this thread's share of the CFL maxima.
// t is the step's start time (time-dependent sources).
// STAGED: s.U and s.B already hold the tile (TMA).
template <typename T, bool CG, bool STAGED = false>
__device__ __forceinline__ void flux_tile(const Geom<T>& g, const Phys<T>& p, const T* U, const T* __restrict__ B,
                                          T* Lout, T* Sout, int x0, int y0, SmemFlux<T>& s, double t, T& mx, T& my) {
  const int tid = threadIdx.x;
  const int nvx = min(TX, g.gc + g.nx - x0), nvy = min(TY, g.gc + g.ny - y0);

  if constexpr (!STAGED) {
    for (int idx = tid; idx < HX * HY; idx += NT) {
      const int lx = idx % HX, ly = idx / HX;
      const int gx = x0 - 2 + lx, gy = y0 - 2 + ly;
      const bool ok = gx < g.N1 && gy < g.N2;
      const long long o = sidx(g, gx, gy);
#pragma unroll
      for (int k = 0; k < 3; ++k) s.U[k * HX * HY + idx] = ok ? gld<CG>(U + k * g.PS + o) : (T)0;
    }
    if (!g.bottom_const) load_corners(g, B, s.B, x0, y0);
  }
  if (p.any_dynamic && tid == 0) point_scalars<T>(p, t, s.scal);
  __syncthreads();

  BTile<T> bt{s.B, g.bottom_const, g.bconst};
  T acc[CPT][3];
  tile_derivative<T, true>(p, s.U, bt, s.L, s.R, s.F, acc, mx, my, nvx, nvy);

#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    const int c = tid + k * NT;
    const int lx = c % TX, ly = c / TX;
    if (lx >= nvx || ly >= nvy) continue;
    const long long o = sidx(g, x0 + lx, y0 + ly);
    acc[k][0] = p.any_dynamic ? add_point_sources<T>(p, acc[k][0], s.scal, o) : add_point_sources<T>(p, acc[k][0]);
#pragma unroll
    for (int j = 0; j < 3; ++j) Lout[j * g.PS + o] = acc[k][j];
    if (p.friction) {
      const int ci = (ly + 2) * HX + lx + 2;
      Sout[o] = friction_factor<T>(p, s.U[ci], s.U[HX * HY + ci], s.U[2 * HX * HY + ci], bt.cell(lx, ly));
    }
  }
}

// Block maximum of per-thread CFL speed keys (IEEE bit patterns of speeds
// >= 0): warp shuffles, then one shared-memory pass; valid in thread 0.
__device__ __forceinline__ void block_key_max(unsigned long long kx, unsigned long long ky,
                                              unsigned long long (*red)[NT / 32], unsigned long long& kx_out,
                                              unsigned long long& ky_out) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    kx = max(kx, __shfl_xor_sync(0xffffffffu, kx, o));
    ky = max(ky, __shfl_xor_sync(0xffffffffu, ky, o));
  }
  if ((tid & 31) == 0) {
    red[0][tid >> 5] = kx;
    red[1][tid >> 5] = ky;
  }
  __syncthreads();
  if (tid == 0) {
    kx = 0;
    ky = 0;
    for (int w = 0; w < NT / 32; ++w) {
      kx = max(kx, red[0][w]);
      ky = max(ky, red[1][w]);
    }
    kx_out = kx;
    ky_out = ky;
  }
}

template <typename T>
__device__ __forceinline__ void block_speed_keys(T mx, T my, unsigned long long (*red)[NT / 32],
                                                 unsigned long long& kx_out, unsigned long long& ky_out) {
  block_key_max(speed_key<T>(mx), speed_key<T>(my), red, kx_out, ky_out);
}

template <typename T>
__global__ void __launch_bounds__(NT, VF_TILE_MIN_BLOCKS) k_flux(Geom<T> g, Phys<T> p, const T* __restrict__ U, const T* __restrict__ B,
                                             T* __restrict__ Lout, T* __restrict__ Sout, StepRecord* rec, int parity) {
  if (!rec->active[parity]) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemFlux<T>& s = *reinterpret_cast<SmemFlux<T>*>(smem_raw);
  const int x0 = g.gc + blockIdx.x * TX, y0 = g.gc + blockIdx.y * TY;
  const double t = p.any_dynamic ? rec->t[parity] : 0.0;
  T mx = (T)0, my = (T)0;
  flux_tile<T, false>(g, p, U, B, Lout, Sout, x0, y0, s, t, mx, my);

  // CFL maxima: warp shuffle, then one atomic per block and direction.
  unsigned long long kx = 0, ky = 0;
  block_speed_keys<T>(mx, my, s.red, kx, ky);
  if (threadIdx.x == 0) {
    atomicMax(&rec->speed_bits[parity][0], kx);
    atomicMax(&rec->speed_bits[parity][1], ky);
  }
}

// Bytes of one staged tile of n planes, and of the corner tile.
template <typename T>
__host__ __device__ constexpr unsigned tile_bytes(int planes) { return (unsigned)(planes * HX * HY * sizeof(T)); }
template <typename T>
__host__ __device__ constexpr unsigned corner_bytes() { return (unsigned)(BHX * BHY * sizeof(T)); }

// k_flux with the tile staged by TMA (Float64). Thread 0 issues one 3D copy of
// the three state planes and one 2D copy of the corners; everyone waits on the
// mbarrier, then the flux pass runs as in k_flux.
template <typename T>
__global__ void __launch_bounds__(NT, VF_TILE_MIN_BLOCKS)
    k_flux_tma(Geom<T> g, Phys<T> p, const __grid_constant__ CUtensorMap mU, const __grid_constant__ CUtensorMap mB,
               const T* __restrict__ U, const T* __restrict__ B, T* __restrict__ Lout, T* __restrict__ Sout,
               StepRecord* rec, int parity) {
  static_assert(sizeof(T) == 8, "TMA tiles are Float64 (the tile origin is 16-byte aligned only for 8-byte cells)");
  if (!rec->active[parity]) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemFlux<T>& s = *reinterpret_cast<SmemFlux<T>*>(smem_raw);
  const int x0 = g.gc + blockIdx.x * TX, y0 = g.gc + blockIdx.y * TY;
  const int cx = x0 - 2 + XOFF, cy = y0 - 2;
  if (threadIdx.x == 0) {
    const bool ok = tma_ok(cx, (int)sizeof(T), s.U) && (g.bottom_const || tma_ok(cx, (int)sizeof(T), s.B));
    s.plain = ok ? 0 : 1;
    if (ok) {
      mbar_init(&s.bar, 1);
      mbar_expect_tx(&s.bar, tile_bytes<T>(3) + (g.bottom_const ? 0u : corner_bytes<T>()));
      tma_load_3d(s.U, &mU, cx, cy, 0, &s.bar);
      if (!g.bottom_const) tma_load_2d(s.B, &mB, cx, cy, &s.bar);
    }
  }
  __syncthreads();
  if (!s.plain && !mbar_wait_bounded(&s.bar, 0)) {
    rec->wait_fault = 1;
    s.plain = 2;  // gave up; every thread that gives up sets it, the barrier below makes it uniform
  }
  __syncthreads();
  const double t = p.any_dynamic ? rec->t[parity] : 0.0;
  T mx = (T)0, my = (T)0;
  if (s.plain)
    flux_tile<T, false, false>(g, p, U, B, Lout, Sout, x0, y0, s, t, mx, my);
  else
    flux_tile<T, false, true>(g, p, U, B, Lout, Sout, x0, y0, s, t, mx, my);

  unsigned long long kx = 0, ky = 0;
  block_speed_keys<T>(mx, my, s.red, kx, ky);
  if (threadIdx.x == 0) {
    atomicMax(&rec->speed_bits[parity][0], kx);
    atomicMax(&rec->speed_bits[parity][1], ky);
  }
  // After a give-up, wait once more (bounded) so a late copy does not land
  // after the block has released its shared memory.
  if (s.plain == 2 && threadIdx.x == 0) mbar_wait_bounded(&s.bar, 0);
}

// dt of stage 1 from the CFL maxima, src/simulator.jl:147-150.
template <typename T>
__device__ __forceinline__ double cfl_dt(const Geom<T>& g, double ax, double ay, double max_dt) {
  double dt = jmin<double>(g.cfl * jmin<double>(g.dx / ax, g.dy / ay), max_dt);
  if (sizeof(T) == 4) dt = (double)(float)dt;  // current_timestep is a MVector{1,Float32}
  return dt;
}

// The simulated time after a step (t += dt, src/simulator.jl:205, in the
// backend's real type).
template <typename T>
__device__ __forceinline__ double next_time(double t, double dt) {
  return sizeof(T) == 4 ? (double)((float)t + (float)dt) : t + dt;
}

// max_dt of simulate_to_time (src/simulator.jl:199-203).
__device__ __forceinline__ double loop_max_dt(int match_endtime, double endtime, double t, int has_max_ts,
                                              double max_ts) {
  double max_dt = match_endtime ? endtime - t : __longlong_as_double(0x7ff0000000000000ll);
  if (has_max_ts) max_dt = jmin<double>(max_dt, max_ts);
  return max_dt;
}

// dt and time bookkeeping of the step of this parity.
template <typename T>
__device__ __forceinline__ double step_dt(const Geom<T>& g, const StepRecord* rec, int parity) {
  if (rec->force_dt) return rec->forced_dt;
  const double ax = speed_from_key<T>(rec->speed_bits[parity][0]);
  const double ay = speed_from_key<T>(rec->speed_bits[parity][1]);
  const double max_dt = rec->explicit_mode
                            ? rec->explicit_max_dt
                            : loop_max_dt(rec->match_endtime, rec->endtime, rec->t[parity], rec->has_max_ts,
                                          rec->max_ts);
  return cfl_dt<T>(g, ax, ay, max_dt);
}

template <typename T>
__device__ __forceinline__ void advance_record(StepRecord* rec, int parity, double dt) {
  const double tn = next_time<T>(rec->t[parity], dt);
  rec->last_dt = dt;
  rec->t[parity ^ 1] = tn;
  rec->n_done += 1;
  const bool more = !rec->explicit_mode && (tn < rec->endtime) && !(tn + dt >= rec->stop_time);
  rec->active[parity ^ 1] = more ? 1 : 0;
  rec->speed_bits[parity ^ 1][0] = 0ull;
  rec->speed_bits[parity ^ 1][1] = 0ull;
}

__device__ __forceinline__ void carry_record(StepRecord* rec, int parity) {
  rec->t[parity ^ 1] = rec->t[parity];
  rec->active[parity ^ 1] = 0;
}

// Ghosts written by the owner of each boundary source cell: wall mirrors
// (src/bc.jl:81-110; x ghosts negate hu, y ghosts hv) or periodic copies
// (src/bc.jl:29-40). Corner ghosts are never written, as in the reference.
// INTERIOR = false: the ghost copies only (the cell itself is stored elsewhere).
template <typename T, bool INTERIOR = true>
__device__ __forceinline__ void store_with_ghosts(const Geom<T>& g, T* __restrict__ Uo, int gx, int gy, T w, T hu,
                                                  T hv) {
  if constexpr (INTERIOR) {
    const long long o = sidx(g, gx, gy);
    Uo[o] = w;
    Uo[g.PS + o] = hu;
    Uo[2 * g.PS + o] = hv;
  }
  int gxs[2] = {-1, -1}, gys[2] = {-1, -1};
  const T sx = g.bc == 1 ? (T)-1 : (T)1;  // normal momentum sign across a ghost
  if (g.bc == 2) {
    if (gx < 2 * g.gc) gxs[0] = gx + g.nx;
    if (gx >= g.nx) gxs[1] = gx - g.nx;
    if (gy < 2 * g.gc) gys[0] = gy + g.ny;
    if (gy >= g.ny) gys[1] = gy - g.ny;
  } else if (g.bc == 3) {  // Neumann: left mirror, bottom from the top rows
    const int lo = g.gc;
    if (gx == lo) gxs[0] = lo - 1;
    if (gx == lo + 1) gxs[0] = lo - 2;
    if (gy >= g.ny) gys[1] = gy - g.ny;
  } else {
    const int lo = g.gc, hi = g.gc + g.nx - 1;
    if (gx == lo) gxs[0] = lo - 1;
    if (gx == lo + 1) gxs[0] = lo - 2;
    if (gx == hi) gxs[1] = hi + 1;
    if (gx == hi - 1) gxs[1] = hi + 2;
    const int ylo = g.gc, yhi = g.gc + g.ny - 1;
    if (gy == ylo) gys[0] = ylo - 1;
    if (gy == ylo + 1) gys[0] = ylo - 2;
    if (gy == yhi) gys[1] = yhi + 1;
    if (gy == yhi - 1) gys[1] = yhi + 2;
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    if (gxs[i] >= 0) {
      const long long q = sidx(g, gxs[i], gy);
      Uo[q] = w;
      Uo[g.PS + q] = sx * hu;
      Uo[2 * g.PS + q] = hv;
    }
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    if (gys[i] >= 0) {
      const long long q = sidx(g, gx, gys[i]);
      Uo[q] = w;
      Uo[g.PS + q] = hu;
      Uo[2 * g.PS + q] = sx * hv;
    }
  }
}

// Stage-1 pointwise update of one cell: Euler, friction, dry clamp.
// src/timestepper/rungekutta.jl:39-41, src/friction.jl:77,80-84,
// src/timestepper/timestepper.jl:41-51.
template <typename T>
__device__ __forceinline__ void stage1_point(const Phys<T>& p, T tdt, T u0, T u1, T u2, T l0, T l1, T l2, T S, T Bc,
                                             T& w, T& hu, T& hv) {
  w = u0 + tdt * l0;
  hu = u1 + tdt * l1;
  hv = u2 + tdt * l2;
  if (p.friction) apply_friction<T>(tdt, S, hu, hv);
  dry_clamp<T>(p, w, hu, hv, Bc);
}

// NeumannBC's right and top ghosts (src/bc.jl:53,58 copy ghost onto ghost):
// the outer ghost of a row or column evolves by the all-cell passes alone --
// no flux, its rain and infiltration, its own friction and dry clamp -- and
// the boundary update copies it onto the inner ghost. (x, y) is the outer
// ghost; its stage-1 value, and with rk2 its stage-2 value, is written to it
// and to the inner ghost (x-1, y) or (x, y-1). scal holds point_scalars().
template <typename T, bool CG>
__device__ __forceinline__ void neumann_u1(const Geom<T>& g, const Phys<T>& p, T tdt, const T* U0,
                                           const T* __restrict__ B, const T* scal, int x, int y, T& w, T& hu, T& hv,
                                           T& a0, T& a1, T& a2, T& lpt, T& Bc) {
  const long long o = sidx(g, x, y);
  Bc = g.bconst;
  if (!g.bottom_const) {
    const long long b = (long long)y * g.PB + x + XOFF;
    Bc = (T)0.25 * (((B[b] + B[b + 1]) + B[b + g.PB]) + B[b + g.PB + 1]);
  }
  a0 = gld<CG>(U0 + o);
  a1 = gld<CG>(U0 + g.PS + o);
  a2 = gld<CG>(U0 + 2 * g.PS + o);
  lpt = p.any_dynamic ? add_point_sources<T>(p, (T)0, scal, o) : add_point_sources<T>(p, (T)0);
  T S = (T)0;
  if (p.friction && friction_active<T>(a1, a2)) S = friction_factor<T>(p, a0, a1, a2, Bc);
  stage1_point<T>(p, tdt, a0, a1, a2, lpt, (T)0, (T)0, S, Bc, w, hu, hv);
}

template <typename T, bool CG>
__device__ __forceinline__ void neumann_outer(const Geom<T>& g, const Phys<T>& p, T tdt, const T* U0,
                                              const T* __restrict__ B, const T* scal, int x, int y, int axis, bool rk2,
                                              T* Uo) {
  T w, hu, hv, a0, a1, a2, lpt, Bc;
  neumann_u1<T, CG>(g, p, tdt, U0, B, scal, x, y, w, hu, hv, a0, a1, a2, lpt, Bc);
  if (rk2) {  // src/timestepper/rungekutta.jl:42-50 on the ghost
    const T v0 = w, v1 = hu, v2 = hv;
    w = v0 + tdt * lpt;
    hu = v1 + tdt * (T)0;
    hv = v2 + tdt * (T)0;
    w = (T)0.5 * (a0 + w);
    hu = (T)0.5 * (a1 + hu);
    hv = (T)0.5 * (a2 + hv);
    if (p.friction && friction_active<T>(v1, v2)) apply_friction<T>(tdt, friction_factor<T>(p, v0, v1, v2, Bc), hu, hv);
    dry_clamp<T>(p, w, hu, hv, Bc);
  }
  const long long q0 = sidx(g, x, y);
  const long long q1 = axis == 0 ? sidx(g, x - 1, y) : sidx(g, x, y - 1);
  Uo[q0] = w;
  Uo[g.PS + q0] = hu;
  Uo[2 * g.PS + q0] = hv;
  Uo[q1] = w;
  Uo[g.PS + q1] = hu;
  Uo[2 * g.PS + q1] = hv;
}

// ---------------------------------------------------------------------------
// RK2 stage pass.
// L, R and F come first and are contiguous: before the stage-2 derivative
// overwrites them they hold the TMA-staged halo tiles of U0 (3 planes), L (3)
// and S (1), STAGE_PLANES planes of HX x HY from offset 0 (k_stage2_tma).
// For Float64 every TMA destination starts 128-byte aligned.
template <typename T>
struct SmemStage {
  T L[3 * LRN];
  T R[3 * LRN];
  T F[3 * FN];
  T U1[3 * HX * HY];
  T U0[3 * TX * TY];
  T B[BHX * BHY];
  double dt;
  T scal[8];
  unsigned long long bar;  // mbarrier of the tile copies
  int plain;               // 0: staged by TMA; 1: not staged (alignment); 2: the wait gave up
};
constexpr int STAGE_PLANES = 7;
static_assert(3 * LRN + 3 * LRN + 3 * FN >= STAGE_PLANES * HX * HY, "stage staging area must fit in L, R, F");

// RK2 stage pass over one tile at (x0, y0) (block-collective): U2 with its
// ghosts into Uo. dt is the step's dt, t its start time.
// STAGED: the halo tiles of U0, L, S sit at the start of s (planes of HX x HY:
// U0 0..2, L 3..5, S 6) and s.B holds the corners (TMA); the interior of U2
// goes to s.U0 (in place: each thread overwrites the cells it read) for a
// tensor store by the caller, its ghost copies straight to Uo.
template <typename T, bool CG, bool STAGED = false>
__device__ __forceinline__ void stage2_tile(const Geom<T>& g, const Phys<T>& p, const T* U0, const T* __restrict__ B,
                                            const T* Lin, const T* Sin, T* Uo, int x0, int y0, SmemStage<T>& s,
                                            double dt, double t) {
  const int tid = threadIdx.x;
  const int nvx = min(TX, g.gc + g.nx - x0), nvy = min(TY, g.gc + g.ny - y0);
  if (p.any_dynamic && tid == 1) point_scalars<T>(p, t, s.scal);
  if (!STAGED && !g.bottom_const) load_corners(g, B, s.B, x0, y0);
  __syncthreads();
  const T* stg = s.L;  // staged planes (STAGED only)
  const T tdt = (T)dt;
  BTile<T> bt{s.B, g.bottom_const, g.bconst};

  // U1 on tile + halo, from U0, L, S. Ghost cells take U1 of their boundary
  // source cell (src/bc.jl:29-40, 81-110), computed the same pointwise way;
  // corner ghosts are never read and stay zero.
  for (int idx = tid; idx < HX * HY; idx += NT) {
    const int lx = idx % HX - 2, ly = idx / HX - 2;
    const int gx = x0 + lx, gy = y0 + ly;
    const bool xin = gx >= g.gc && gx < g.gc + g.nx;
    const bool yin = gy >= g.gc && gy < g.gc + g.ny;
    T w = (T)0, hu = (T)0, hv = (T)0;
    if (xin && yin) {
      T a0, a1, a2, l0, l1, l2, S;
      if constexpr (STAGED) {
        constexpr int A = HX * HY;
        a0 = stg[idx];
        a1 = stg[A + idx];
        a2 = stg[2 * A + idx];
        l0 = stg[3 * A + idx];
        l1 = stg[4 * A + idx];
        l2 = stg[5 * A + idx];
        S = p.friction ? stg[6 * A + idx] : (T)0;
      } else {
        const long long o = sidx(g, gx, gy);
        a0 = gld<CG>(U0 + o);
        a1 = gld<CG>(U0 + g.PS + o);
        a2 = gld<CG>(U0 + 2 * g.PS + o);
        l0 = gld<CG>(Lin + o);
        l1 = gld<CG>(Lin + g.PS + o);
        l2 = gld<CG>(Lin + 2 * g.PS + o);
        S = p.friction ? gld<CG>(Sin + o) : (T)0;
      }
      stage1_point<T>(p, tdt, a0, a1, a2, l0, l1, l2, S, bt.cell(lx, ly), w, hu, hv);
      if (lx >= 0 && lx < TX && ly >= 0 && ly < TY) {
        const int t = ly * TX + lx;
        s.U0[t] = a0;
        s.U0[TX * TY + t] = a1;
        s.U0[2 * TX * TY + t] = a2;
      }
    } else if (yin && gx < g.N1) {
      if (g.bc == 3 && gx >= g.gc + g.nx) {
        T a0, a1, a2, lpt, Bg;
        neumann_u1<T, CG>(g, p, tdt, U0, B, s.scal, g.N1 - 1, gy, w, hu, hv, a0, a1, a2, lpt, Bg);
      } else {
        u1_global<T, CG>(g, p, tdt, U0, Lin, Sin, B, bc_source(gx, g.gc, g.nx, g.bc, 0), gy, w, hu, hv);
        if (g.bc == 1) hu = -hu;
      }
    } else if (xin && gy < g.N2) {
      if (g.bc == 3 && gy >= g.gc + g.ny) {
        T a0, a1, a2, lpt, Bg;
        neumann_u1<T, CG>(g, p, tdt, U0, B, s.scal, gx, g.N2 - 1, w, hu, hv, a0, a1, a2, lpt, Bg);
      } else {
        u1_global<T, CG>(g, p, tdt, U0, Lin, Sin, B, gx, bc_source(gy, g.gc, g.ny, g.bc, 1), w, hu, hv);
        if (g.bc == 1) hv = -hv;
      }
    }
    s.U1[idx] = w;
    s.U1[HX * HY + idx] = hu;
    s.U1[2 * HX * HY + idx] = hv;
  }
  __syncthreads();

  T acc[CPT][3];
  T mx = (T)0, my = (T)0;
  tile_derivative<T, false>(p, s.U1, bt, s.L, s.R, s.F, acc, mx, my, nvx, nvy);

#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    const int c = tid + k * NT;
    const int lx = c % TX, ly = c / TX;
    if (lx >= nvx || ly >= nvy) continue;
    const long long o = sidx(g, x0 + lx, y0 + ly);
    acc[k][0] = p.any_dynamic ? add_point_sources<T>(p, acc[k][0], s.scal, o) : add_point_sources<T>(p, acc[k][0]);
    const int ci = (ly + 2) * HX + lx + 2;
    const T v0 = s.U1[ci], v1 = s.U1[HX * HY + ci], v2 = s.U1[2 * HX * HY + ci];
    T w = v0 + tdt * acc[k][0];
    T hu = v1 + tdt * acc[k][1];
    T hv = v2 + tdt * acc[k][2];
    w = (T)0.5 * (s.U0[c] + w);
    hu = (T)0.5 * (s.U0[TX * TY + c] + hu);
    hv = (T)0.5 * (s.U0[2 * TX * TY + c] + hv);
    const T Bc = bt.cell(lx, ly);
    if (p.friction && friction_active<T>(v1, v2)) apply_friction<T>(tdt, friction_factor<T>(p, v0, v1, v2, Bc), hu, hv);
    dry_clamp<T>(p, w, hu, hv, Bc);
    if (STAGED && x0 + lx + XOFF < tma_store_cols(XOFF + g.gc + g.nx)) {
      s.U0[c] = w;  // stored by the tile's tensor store
      s.U0[TX * TY + c] = hu;
      s.U0[2 * TX * TY + c] = hv;
      store_with_ghosts<T, false>(g, Uo, x0 + lx, y0 + ly, w, hu, hv);
    } else {
      store_with_ghosts<T>(g, Uo, x0 + lx, y0 + ly, w, hu, hv);
    }
    if (g.bc == 3) {
      if (x0 + lx == g.gc + g.nx - 1) neumann_outer<T, CG>(g, p, tdt, U0, B, s.scal, g.N1 - 1, y0 + ly, 0, true, Uo);
      if (y0 + ly == g.gc + g.ny - 1) neumann_outer<T, CG>(g, p, tdt, U0, B, s.scal, x0 + lx, g.N2 - 1, 1, true, Uo);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(NT, VF_TILE_MIN_BLOCKS) k_stage2(Geom<T> g, Phys<T> p, const T* __restrict__ U0, const T* __restrict__ B,
                                               const T* __restrict__ Lin, const T* __restrict__ Sin, T* __restrict__ Uo,
                                               StepRecord* rec, int parity) {
  const bool root = blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0;
  if (!rec->active[parity]) {
    if (root) carry_record(rec, parity);
    return;
  }
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemStage<T>& s = *reinterpret_cast<SmemStage<T>*>(smem_raw);
  const int x0 = g.gc + blockIdx.x * TX, y0 = g.gc + blockIdx.y * TY;
  if (threadIdx.x == 0) s.dt = step_dt<T>(g, rec, parity);
  __syncthreads();
  const double dt = s.dt;
  stage2_tile<T, false>(g, p, U0, B, Lin, Sin, Uo, x0, y0, s, dt, rec->t[parity]);
  if (root) advance_record<T>(rec, parity, dt);
}

// k_stage2 with the halo tiles of U0, L, S and the corners staged by TMA
// (Float64): three or four copies on one mbarrier, issued by thread 0.
template <typename T>
__global__ void __launch_bounds__(NT, VF_TILE_MIN_BLOCKS)
    k_stage2_tma(Geom<T> g, Phys<T> p, const __grid_constant__ CUtensorMap mU, const __grid_constant__ CUtensorMap mL,
                 const __grid_constant__ CUtensorMap mS, const __grid_constant__ CUtensorMap mB,
                 const __grid_constant__ CUtensorMap mUo,
                 const T* __restrict__ U0, const T* __restrict__ B, const T* __restrict__ Lin,
                 const T* __restrict__ Sin, T* __restrict__ Uo, StepRecord* rec, int parity) {
  static_assert(sizeof(T) == 8, "TMA tiles are Float64 (the tile origin is 16-byte aligned only for 8-byte cells)");
  const bool root = blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0;
  if (!rec->active[parity]) {
    if (root) carry_record(rec, parity);
    return;
  }
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemStage<T>& s = *reinterpret_cast<SmemStage<T>*>(smem_raw);
  const int x0 = g.gc + blockIdx.x * TX, y0 = g.gc + blockIdx.y * TY;
  const int cx = x0 - 2 + XOFF, cy = y0 - 2;
  if (threadIdx.x == 0) {
    constexpr int A = HX * HY;
    T* stg = s.L;
    const bool ok = tma_ok(cx, (int)sizeof(T), stg) && tma_ok(cx, (int)sizeof(T), stg + 3 * A) &&
                    tma_ok(cx, (int)sizeof(T), stg + 6 * A) && (g.bottom_const || tma_ok(cx, (int)sizeof(T), s.B)) &&
                    tma_ok(x0 + XOFF, (int)sizeof(T), s.U0);
    s.plain = ok ? 0 : 1;
    if (ok) {
      mbar_init(&s.bar, 1);
      mbar_expect_tx(&s.bar, tile_bytes<T>(6) + (p.friction ? tile_bytes<T>(1) : 0u) +
                                 (g.bottom_const ? 0u : corner_bytes<T>()));
      tma_load_3d(stg, &mU, cx, cy, 0, &s.bar);
      tma_load_3d(stg + 3 * A, &mL, cx, cy, 0, &s.bar);
      if (p.friction) tma_load_2d(stg + 6 * A, &mS, cx, cy, &s.bar);
      if (!g.bottom_const) tma_load_2d(s.B, &mB, cx, cy, &s.bar);
    }
    s.dt = step_dt<T>(g, rec, parity);
  }
  __syncthreads();
  if (!s.plain && !mbar_wait_bounded(&s.bar, 0)) {
    rec->wait_fault = 1;
    s.plain = 2;  // gave up
  }
  __syncthreads();
  const double dt = s.dt;
  if (s.plain) {
    stage2_tile<T, false, false>(g, p, U0, B, Lin, Sin, Uo, x0, y0, s, dt, rec->t[parity]);
  } else {
    stage2_tile<T, false, true>(g, p, U0, B, Lin, Sin, Uo, x0, y0, s, dt, rec->t[parity]);
    // The interior tile from s.U0 (128-byte aligned, x0 + XOFF even) in one tensor store.
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_store_3d(&mUo, s.U0, x0 + XOFF, y0, 0);
      bulk_commit();
      bulk_wait_all();
    }
  }
  if (root) advance_record<T>(rec, parity, dt);
  if (s.plain == 2 && threadIdx.x == 0) mbar_wait_bounded(&s.bar, 0);  // a late copy lands before exit
}

// ---------------------------------------------------------------------------
// Forward-Euler apply pass: U1 = clamp((U0 + dt*L) ./ (1 .- dt*[0,S,S])).
// Forward-Euler apply over one tile at (x0, y0): the pointwise stage-1 update.
template <typename T, bool CG>
__device__ __forceinline__ void apply_fe_tile(const Geom<T>& g, const Phys<T>& p, const T* U0,
                                              const T* __restrict__ B, const T* Lin, const T* Sin, T* Uo, int x0,
                                              int y0, double dt, double t) {
  const T tdt = (T)dt;
  const int lx = threadIdx.x % TX, ly0 = threadIdx.x / TX;
  for (int ly = ly0; ly < TY; ly += NT / TX) {
    const int gx = x0 + lx, gy = y0 + ly;
    if (gx >= g.gc + g.nx || gy >= g.gc + g.ny) continue;
    const long long o = sidx(g, gx, gy);
    T Bc = g.bconst;
    if (!g.bottom_const) {
      const long long b = (long long)gy * g.PB + gx + XOFF;
      Bc = (T)0.25 * (((B[b] + B[b + 1]) + B[b + g.PB]) + B[b + g.PB + 1]);
    }
    const T S = p.friction ? gld<CG>(Sin + o) : (T)0;
    T w, hu, hv;
    stage1_point<T>(p, tdt, gld<CG>(U0 + o), gld<CG>(U0 + g.PS + o), gld<CG>(U0 + 2 * g.PS + o), gld<CG>(Lin + o),
                    gld<CG>(Lin + g.PS + o), gld<CG>(Lin + 2 * g.PS + o), S, Bc, w, hu, hv);
    store_with_ghosts<T>(g, Uo, gx, gy, w, hu, hv);
    if (g.bc == 3 && (gx == g.gc + g.nx - 1 || gy == g.gc + g.ny - 1)) {
      T scal[8];
      if (p.any_dynamic) point_scalars<T>(p, t, scal);
      if (gx == g.gc + g.nx - 1) neumann_outer<T, CG>(g, p, tdt, U0, B, scal, g.N1 - 1, gy, 0, false, Uo);
      if (gy == g.gc + g.ny - 1) neumann_outer<T, CG>(g, p, tdt, U0, B, scal, gx, g.N2 - 1, 1, false, Uo);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(NT) k_apply_fe(Geom<T> g, Phys<T> p, const T* __restrict__ U0,
                                                 const T* __restrict__ B, const T* __restrict__ Lin,
                                                 const T* __restrict__ Sin, T* __restrict__ Uo, StepRecord* rec,
                                                 int parity) {
  const bool root = blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0;
  if (!rec->active[parity]) {
    if (root) carry_record(rec, parity);
    return;
  }
  __shared__ double sdt;
  if (threadIdx.x == 0) sdt = step_dt<T>(g, rec, parity);
  __syncthreads();
  const double dt = sdt;
  apply_fe_tile<T, false>(g, p, U0, B, Lin, Sin, Uo, g.gc + blockIdx.x * TX, g.gc + blockIdx.y * TY, dt,
                          rec->t[parity]);
  if (root) advance_record<T>(rec, parity, dt);
}

// Boundary update of a whole volume (after uploads): wall, src/bc.jl:81-110,
// periodic, src/bc.jl:29-40, or Neumann, src/bc.jl:49-60 (right and top: the
// inner ghost takes the outer ghost's value). Ghost columns at interior rows,
// ghost rows at interior columns; corners untouched.
template <typename T>
__global__ void k_bc(Geom<T> g, T* __restrict__ U) {
  const int n_x = g.ny * 2 * g.gc;
  const int n_y = g.nx * 2 * g.gc;
  const T sgn = g.bc == 1 ? (T)-1 : (T)1;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n_x + n_y; idx += gridDim.x * blockDim.x) {
    if (idx < n_x) {
      const int j = g.gc + idx / (2 * g.gc), r = idx % (2 * g.gc);
      const int gx = r < g.gc ? r : g.gc + g.nx + (r - g.gc);
      if (g.bc == 3 && gx >= g.gc + g.nx) {
        if (gx == g.N1 - 2) {
          const long long d = sidx(g, gx, j), sI = sidx(g, g.N1 - 1, j);
          U[d] = U[sI];
          U[g.PS + d] = U[g.PS + sI];
          U[2 * g.PS + d] = U[2 * g.PS + sI];
        }
        continue;
      }
      const int sx = bc_source(gx, g.gc, g.nx, g.bc, 0);
      const long long d = sidx(g, gx, j), sI = sidx(g, sx, j);
      U[d] = U[sI];
      U[g.PS + d] = sgn * U[g.PS + sI];
      U[2 * g.PS + d] = U[2 * g.PS + sI];
    } else {
      const int q = idx - n_x;
      const int i = g.gc + q / (2 * g.gc), r = q % (2 * g.gc);
      const int gy = r < g.gc ? r : g.gc + g.ny + (r - g.gc);
      if (g.bc == 3 && gy >= g.gc + g.ny) {
        if (gy == g.N2 - 2) {
          const long long d = sidx(g, i, gy), sI = sidx(g, i, g.N2 - 1);
          U[d] = U[sI];
          U[g.PS + d] = U[g.PS + sI];
          U[2 * g.PS + d] = U[2 * g.PS + sI];
        }
        continue;
      }
      const int sy = bc_source(gy, g.gc, g.ny, g.bc, 1);
      const long long d = sidx(g, i, gy), sI = sidx(g, i, sy);
      U[d] = U[sI];
      U[g.PS + d] = U[g.PS + sI];
      U[2 * g.PS + d] = sgn * U[2 * g.PS + sI];
    }
  }
}

// State of n interior cells (0-based (i, j) pairs) gathered into out[3][n].
template <typename T>
__global__ void k_sample(Geom<T> g, const T* __restrict__ U, const int* __restrict__ ij, int n, T* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long long o = sidx(g, g.gc + ij[k], g.gc + ij[n + k]);
  out[k] = U[o];
  out[n + k] = U[g.PS + o];
  out[2 * n + k] = U[2 * g.PS + o];
}

// Water volume sum((w - B_cell) * dx * dy) over the interior, in Float64:
// per-block partial sums in a fixed order, then one block sums the partials.
template <typename T>
__global__ void k_volume_partial(Geom<T> g, const T* __restrict__ U, const T* __restrict__ B, double* partial) {
  __shared__ double red[NT];
  double acc = 0.0;
  const long long n = (long long)g.nx * g.ny;
  for (long long c = (long long)blockIdx.x * NT + threadIdx.x; c < n; c += (long long)gridDim.x * NT) {
    const int i = g.gc + (int)(c % g.nx), j = g.gc + (int)(c / g.nx);
    double Bc = (double)g.bconst;
    if (!g.bottom_const) {
      const long long b = (long long)j * g.PB + i + XOFF;
      Bc = (double)((T)0.25 * (((B[b] + B[b + 1]) + B[b + g.PB]) + B[b + g.PB + 1]));
    }
    acc += ((double)U[sidx(g, i, j)] - Bc) * g.dx * g.dy;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}



}  // namespace vf
