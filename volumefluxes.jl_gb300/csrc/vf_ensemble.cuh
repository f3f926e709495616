// vf_ensemble.cuh -- many independent simulations in one launch.
//
// Each scenario (one simulate_to_time of src/simulator.jl:199-212 on its own
// grid, terrain, sources and end time) is owned by one thread-block cluster of
// C CTAs for its whole time loop:
//   flux phase   the cluster's CTAs take the scenario's 32x16 tiles round-robin
//                (tile = rank, rank + C, ...) and run the flux pass of the
//                plain step (L(U0), S(U0), CFL maxima);
//   dt           each CTA publishes its block maxima in shared memory, a
//                hardware cluster barrier (release/acquire) follows, and every
//                CTA reads all C slots through distributed shared memory and
//                computes the same dt, exactly as the plain path does from its
//                atomics (the maximum of IEEE bit patterns is order-free);
//   stage phase  the RK2 stage pass (or the forward-Euler update) per tile,
//                then a second cluster barrier publishes U^{n+1}.
// Scenarios advance with their own dt and stop at their own end time, so a
// cluster leaves as soon as its scenario is done and the hardware block
// scheduler starts the next pending cluster in its place: the scenario list is
// a work queue drained by the GPU itself. Nothing waits on another cluster;
// the only waits are the hardware cluster barriers, which every CTA of the
// cluster reaches because the loop control (t, dt, the step count and the
// watchdog flag of rank 0) is identical in all of them.
//
// Step data written inside the launch is read back with ld.global.cg
// (gld<true>), never through the read-only or L1 paths.
#pragma once
#include "vf_march.cuh"

namespace vf {

// Per-scenario status codes (EnsResult::status).
constexpr int kEnsOk = 0;
constexpr int kEnsTimeout = 1;  // the launch's watchdog fired before the end time
constexpr int kEnsStalled = 2;  // t + dt == t in the real type: no progress possible
constexpr int kEnsMaxSteps = 3; // stopped at max_steps

struct EnsResult {
  double t;
  double last_dt;
  long long steps;
  int status;
  int done;  // set last, after a system-scope fence
};

template <typename T>
struct EnsItem {
  Geom<T> g;
  Phys<T> p;
  const T* B;
  T* U[2];  // step n reads U[n & 1] and writes U[(n & 1) ^ 1]
  T* L;
  T* S;
  double t0, endtime, max_ts;
  int match_endtime, has_max_ts, rk2;
  int seg_rows;  // rows per strip segment (column-marching members)
  long long max_steps;
  EnsResult* res;                // host-mapped: the host sees each scenario finish
  unsigned long long* epoch;     // batch start (globaltimer ns), set by the first CTA that runs
};

template <typename T>
union SmemEns {
  SmemFlux<T> f;
  SmemStage<T> s;
};

struct EnsSlot {
  unsigned long long kx, ky;
  int stop;
  int pad_;
};

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cluster_barrier() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::
          : "memory");
}

__device__ __forceinline__ unsigned dsmem_addr(const void* local, unsigned rank) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(local);
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}

__device__ __forceinline__ unsigned long long dsmem_ld_u64(const void* local, unsigned rank) {
  unsigned long long v;
  asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(dsmem_addr(local, rank)) : "memory");
  return v;
}

__device__ __forceinline__ int dsmem_ld_s32(const void* local, unsigned rank) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(dsmem_addr(local, rank)) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Resident CTAs per SM the ensemble kernel is compiled for: two Float64 CTAs
// fill the shared memory (2 x 77 KB); Float32 takes three.
#ifndef VF_ENS_BLOCKS_F32
#define VF_ENS_BLOCKS_F32 3
#endif
template <typename T> struct EnsBlocks { static constexpr int value = sizeof(T) == 8 ? 2 : VF_ENS_BLOCKS_F32; };

// VAR 0: column-marching RK2 phases (vf_march.cuh), each warp taking strip
// segments (strip, seg) = unit % nstrips, unit / nstrips, for units
// rank * 8 + warp, stepping by 8 * C; wall BCs, linear reconstruction and
// constant sources only -- the kernels the plain path runs for such Float32
// simulations. VAR 2: the same flux phase with the forward-Euler update per
// tile. VAR 1: shared-memory tile phases (vf_kernels.cuh), every
// configuration. Each variant is its own kernel so that one's code does not
// change how another is compiled.
template <typename T, int VAR>
__global__ void __launch_bounds__(NT, EnsBlocks<T>::value) k_ensemble(const EnsItem<T>* __restrict__ items,
                                                                      const int* __restrict__ order, int csize,
                                                                      unsigned long long time_limit_ns) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemEns<T>& sm = *reinterpret_cast<SmemEns<T>*>(smem_raw);
  __shared__ EnsItem<T> sit;
  __shared__ EnsSlot slot;
  __shared__ unsigned long long red[2][NT / 32];
  __shared__ double sdt;
  __shared__ int sstop;

  const int tid = threadIdx.x;
  const unsigned rank = cluster_rank();
  {
    const EnsItem<T>* it = items + order[blockIdx.x / csize];
    static_assert(sizeof(EnsItem<T>) % 8 == 0, "EnsItem copies in 8-byte words");
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(it);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sit);
    for (int i = tid; i < (int)(sizeof(EnsItem<T>) / 8); i += NT) dst[i] = src[i];
  }
  __syncthreads();
  const Geom<T>& g = sit.g;
  const Phys<T>& p = sit.p;
  const int tiles_x = (g.nx + TX - 1) / TX;
  const int ntiles = tiles_x * ((g.ny + TY - 1) / TY);
  constexpr int kWarps = NT / 32;
  const int warp = tid >> 5;
  const int seg = sit.seg_rows;
  const int nstrips = (g.nx + MOUT - 1) / MOUT;
  const int nunits = nstrips * ((g.ny + seg - 1) / seg);
  // The watchdog counts from the batch's start, not this cluster's: a
  // simulation that waited for free SMs has less time left.
  __shared__ unsigned long long s_start;
  if (tid == 0) {
    const unsigned long long now = global_ns();
    const unsigned long long prev = atomicCAS(sit.epoch, 0ull, now);
    s_start = prev ? prev : now;
  }
  __syncthreads();
  const unsigned long long t_start = s_start;

  double t = sit.t0, last_dt = 0.0;
  long long n = 0;
  int status = kEnsOk;
  bool go = t < sit.endtime && sit.max_steps > 0;
  while (go) {
    const T* U0 = sit.U[n & 1];
    T* U1 = sit.U[(n & 1) ^ 1];
    unsigned long long kx = 0, ky = 0;
    if constexpr (VAR != 1) {
      unsigned long long mx = 0, my = 0;
      for (int u = (int)rank * kWarps + warp; u < nunits; u += csize * kWarps) {
        StripGeom s;
        strip_setup_at(g, seg, u % nstrips, u / nstrips, s);
        flux_march_unit<T, true>(g, p, U0, sit.B, sit.L, sit.S, s, mx, my);
      }
      block_key_max(mx, my, red, kx, ky);
    } else {
      T mx = (T)0, my = (T)0;
      for (int tile = (int)rank; tile < ntiles; tile += csize) {
        flux_tile<T, true>(g, p, U0, sit.B, sit.L, sit.S, g.gc + (tile % tiles_x) * TX, g.gc + (tile / tiles_x) * TY,
                           sm.f, t, mx, my);
        __syncthreads();
      }
      block_speed_keys<T>(mx, my, red, kx, ky);
    }
    if (tid == 0) {
      slot.kx = kx;
      slot.ky = ky;
      slot.stop = (rank == 0 && global_ns() - t_start > time_limit_ns) ? 1 : 0;
    }
    cluster_barrier();
    if (tid == 0) {
      unsigned long long ax = 0, ay = 0;
      for (int r = 0; r < csize; ++r) {
        ax = max(ax, dsmem_ld_u64(&slot.kx, (unsigned)r));
        ay = max(ay, dsmem_ld_u64(&slot.ky, (unsigned)r));
      }
      sstop = dsmem_ld_s32(&slot.stop, 0u);
      const double max_dt = loop_max_dt(sit.match_endtime, sit.endtime, t, sit.has_max_ts, sit.max_ts);
      sdt = cfl_dt<T>(g, speed_from_key<T>(ax), speed_from_key<T>(ay), max_dt);
    }
    __syncthreads();
    if (sstop) {
      status = kEnsTimeout;
      break;
    }
    const double dt = sdt;
    if constexpr (VAR == 0) {
      for (int u = (int)rank * kWarps + warp; u < nunits; u += csize * kWarps) {
        StripGeom s;
        strip_setup_at(g, seg, u % nstrips, u / nstrips, s);
        stage_march_unit<T, true>(g, p, U0, sit.B, sit.L, sit.S, U1, s, (T)dt);
      }
    } else if constexpr (VAR == 2) {
      for (int tile = (int)rank; tile < ntiles; tile += csize)
        apply_fe_tile<T, true>(g, p, U0, sit.B, sit.L, sit.S, U1, g.gc + (tile % tiles_x) * TX,
                               g.gc + (tile / tiles_x) * TY, dt, t);
    } else {
      for (int tile = (int)rank; tile < ntiles; tile += csize) {
        const int x0 = g.gc + (tile % tiles_x) * TX, y0 = g.gc + (tile / tiles_x) * TY;
        if (sit.rk2) {
          stage2_tile<T, true>(g, p, U0, sit.B, sit.L, sit.S, U1, x0, y0, sm.s, dt, t);
        } else {
          apply_fe_tile<T, true>(g, p, U0, sit.B, sit.L, sit.S, U1, x0, y0, dt, t);
        }
        __syncthreads();
      }
    }
    cluster_barrier();
    const double tn = next_time<T>(t, dt);
    last_dt = dt;
    ++n;
    if (!(tn != t)) {
      t = tn;
      status = kEnsStalled;
      break;
    }
    t = tn;
    go = t < sit.endtime;
    if (go && n >= sit.max_steps) {
      status = kEnsMaxSteps;
      go = false;
    }
  }
  // No CTA may leave while a peer can still read its slot.
  cluster_barrier();
  if (rank == 0 && tid == 0) {
    EnsResult* r = sit.res;
    r->t = t;
    r->last_dt = last_dt;
    r->steps = n;
    r->status = status;
    __threadfence_system();
    *reinterpret_cast<volatile int*>(&r->done) = 1;
  }
}

}  // namespace vf
