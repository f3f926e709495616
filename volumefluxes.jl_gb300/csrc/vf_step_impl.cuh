// vf_step_impl.cuh -- launcher bodies shared by the per-precision units.
#pragma once
#include "vf_launch.cuh"

namespace vf {

static __global__ void k_volume_final_impl(const double* partial, int n, double* out) {
  __shared__ double red[NT];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += NT) acc += partial[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// Rows per marching segment of the flux and of the stage pass. Shorter
// segments recompute more halo rows (4 per segment) but give the block
// scheduler more, smaller units: measured on the Float32 4096^2 step (ms per
// launch), flux 0.351 / 0.334 / 0.326 / 0.323 / 0.327 at 96 / 64 / 48 / 40 /
// 32 rows, stage 0.534 / 0.474 / 0.460 / 0.454 / 0.449 / 0.451 at 96 / 64 /
// 48 / 32 / 24 / 16 rows (the same bits at every length).
template <typename T> struct MarchSeg {
  static constexpr int flux = 40;
  static constexpr int stage = 24;
};

template <typename T>
cudaError_t configure_impl() {
  cudaError_t e = cudaFuncSetAttribute(k_flux<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemFlux<T>));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage2<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemStage<T>));
  if (e != cudaSuccess) return e;
  if constexpr (sizeof(T) == 8) {
    e = cudaFuncSetAttribute(k_flux_tma<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemFlux<T>));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_stage2_tma<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemStage<T>));
    if (e != cudaSuccess) return e;
  }
  e = cudaFuncSetAttribute(k_ensemble<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemEns<T>));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_ensemble<T, 1>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if constexpr (sizeof(T) == 4) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_ensemble<T, 0>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_ensemble<T, 2>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  }
  return e;
}

// Column marching (variants 0 and 2) exists for Float32 only: the Float64
// members run on tiles, where full warps keep the 1/64-rate FP64 pipe busy.
template <typename T, int VAR>
cudaLaunchConfig_t ensemble_config(int n, int csize, cudaStream_t st, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(n * csize), 1, 1);
  cfg.blockDim = dim3(NT, 1, 1);
  cfg.dynamicSmemBytes = VAR == 1 ? sizeof(SmemEns<T>) : 0;  // marching needs none
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <typename T>
cudaError_t launch_ensemble_impl(const EnsItem<T>* items, const int* order, int n, int csize, int variant,
                                 unsigned long long time_limit_ns, cudaStream_t st) {
  cudaLaunchAttribute attr[1];
  if (variant == 0 || variant == 2) {
    if constexpr (sizeof(T) == 8) {
      return cudaErrorInvalidValue;
    } else {
      cudaLaunchConfig_t cfg = ensemble_config<T, 0>(n, csize, st, attr);
      if (variant == 2) return cudaLaunchKernelEx(&cfg, k_ensemble<T, 2>, items, order, csize, time_limit_ns);
      return cudaLaunchKernelEx(&cfg, k_ensemble<T, 0>, items, order, csize, time_limit_ns);
    }
  }
  cudaLaunchConfig_t cfg = ensemble_config<T, 1>(n, csize, st, attr);
  return cudaLaunchKernelEx(&cfg, k_ensemble<T, 1>, items, order, csize, time_limit_ns);
}

template <typename T>
cudaError_t ensemble_max_clusters_impl(int csize, int variant, int* out) {
  cudaLaunchAttribute attr[1];
  if (variant == 0 || variant == 2) {
    if constexpr (sizeof(T) == 8) {
      return cudaErrorInvalidValue;
    } else {
      cudaLaunchConfig_t cfg = ensemble_config<T, 0>(1, csize, nullptr, attr);
      if (variant == 2) return cudaOccupancyMaxActiveClusters(out, k_ensemble<T, 2>, &cfg);
      return cudaOccupancyMaxActiveClusters(out, k_ensemble<T, 0>, &cfg);
    }
  }
  cudaLaunchConfig_t cfg = ensemble_config<T, 1>(1, csize, nullptr, attr);
  return cudaOccupancyMaxActiveClusters(out, k_ensemble<T, 1>, &cfg);
}

template <typename T>
dim3 march_grid(const Geom<T>& g, int seg) {
  const int nstrips = (g.nx + MOUT - 1) / MOUT;
  return dim3((nstrips + MWPB - 1) / MWPB, (g.ny + seg - 1) / seg);
}

// Index of the handle volume Uin is (0 or 1) when the launch can stage its
// tiles with the handle's tensor maps, else -1.
template <typename T>
int tma_volume(const StepArgs<T>& a, const T* Uin) {
  if constexpr (sizeof(T) != 8) {
    return -1;
  } else {
    if (!a.tma.ok || a.variant != 1 || a.L != a.tma.Lb || a.S != a.tma.Sb || a.B != a.tma.Bb) return -1;
    if (Uin == a.tma.Ub[0]) return 0;
    if (Uin == a.tma.Ub[1]) return 1;
    return -1;
  }
}

template <typename T>
cudaError_t launch_flux_impl(const StepArgs<T>& a, const T* Uin, int parity, cudaStream_t st) {
  if constexpr (sizeof(T) == 8) {
    const int v = tma_volume<T>(a, Uin);
    if (v >= 0) {
      const dim3 grid((a.g.nx + TX - 1) / TX, (a.g.ny + TY - 1) / TY);
      k_flux_tma<T><<<grid, NT, sizeof(SmemFlux<T>), st>>>(a.g, a.p, a.tma.U[v], a.tma.B, Uin, a.B, a.L, a.S, a.rec,
                                                            parity);
      return cudaGetLastError();
    }
  }
  if (a.variant == 0) {
    k_flux_march<T, MarchSeg<T>::flux><<<march_grid(a.g, MarchSeg<T>::flux), MW * MWPB, 0, st>>>(
        a.g, a.p, Uin, a.B, a.L, a.S, a.rec, parity);
    return cudaGetLastError();
  }
  const dim3 grid((a.g.nx + TX - 1) / TX, (a.g.ny + TY - 1) / TY);
  k_flux<T><<<grid, NT, sizeof(SmemFlux<T>), st>>>(a.g, a.p, Uin, a.B, a.L, a.S, a.rec, parity);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_stage_impl(const StepArgs<T>& a, const T* Uin, T* Uout, int parity, cudaStream_t st) {
  const dim3 grid((a.g.nx + TX - 1) / TX, (a.g.ny + TY - 1) / TY);
  if (a.rk2 && a.variant == 0) {
    k_stage_march<T, MarchSeg<T>::stage><<<march_grid(a.g, MarchSeg<T>::stage), MW * MWPB, 0, st>>>(
        a.g, a.p, Uin, a.B, a.L, a.S, Uout, a.rec, parity);
  } else if (a.rk2) {
    if constexpr (sizeof(T) == 8) {
      const int v = tma_volume<T>(a, Uin);
      if (v >= 0 && Uout == a.tma.Ub[v ^ 1]) {
        k_stage2_tma<T><<<grid, NT, sizeof(SmemStage<T>), st>>>(a.g, a.p, a.tma.U[v], a.tma.L, a.tma.S, a.tma.B,
                                                                 a.tma.Ust[v ^ 1], Uin, a.B, a.L, a.S, Uout, a.rec,
                                                                 parity);
        return cudaGetLastError();
      }
    }
    k_stage2<T><<<grid, NT, sizeof(SmemStage<T>), st>>>(a.g, a.p, Uin, a.B, a.L, a.S, Uout, a.rec, parity);
  } else {
    k_apply_fe<T><<<grid, NT, 0, st>>>(a.g, a.p, Uin, a.B, a.L, a.S, Uout, a.rec, parity);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_step_impl(const StepArgs<T>& a, const T* Uin, T* Uout, int parity, cudaStream_t st) {
  cudaError_t e = launch_flux_impl<T>(a, Uin, parity, st);
  if (e != cudaSuccess) return e;
  return launch_stage_impl<T>(a, Uin, Uout, parity, st);
}

template <typename T>
cudaError_t launch_bc_impl(const Geom<T>& g, T* U, cudaStream_t st) {
  const int n = 2 * g.gc * (g.nx + g.ny);
  int blocks = (n + NT - 1) / NT;
  if (blocks > 4096) blocks = 4096;
  k_bc<T><<<blocks, NT, 0, st>>>(g, U);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_volume_impl(const Geom<T>& g, const T* U, const T* B, double* partial, int nblocks, double* out,
                               cudaStream_t st) {
  k_volume_partial<T><<<nblocks, NT, 0, st>>>(g, U, B, partial);
  k_volume_final_impl<<<1, NT, 0, st>>>(partial, nblocks, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_point_impl(const AdjArgs<T>& a, int* nblocks_out, cudaStream_t st) {
  const dim3 blk(32, 8);
  const dim3 grid((a.g.nx + 31) / 32, (a.g.ny + 7) / 8);
  k_adj_point<T><<<grid, blk, 0, st>>>(a);
  if (nblocks_out) *nblocks_out = (int)(grid.x * grid.y);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_recon_impl(const AdjArgs<T>& a, int dir, cudaStream_t st) {
  const dim3 blk(32, 4);
  if (dir == 0) {
    const dim3 grid((a.g.nx + 2 + 31) / 32, (a.g.ny + 3) / 4);
    k_adj_recon<T, 0><<<grid, blk, 0, st>>>(a);
  } else {
    const dim3 grid((a.g.ny + 2 + 31) / 32, (a.g.nx + 3) / 4);
    k_adj_recon<T, 1><<<grid, blk, 0, st>>>(a);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_gather_impl(const AdjArgs<T>& a, cudaStream_t st) {
  const dim3 blk(32, 8);
  k_adj_gather<T><<<dim3((a.g.nx + 31) / 32, (a.g.ny + 7) / 8), blk, 0, st>>>(a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_corner_impl(const AdjArgs<T>& a, cudaStream_t st) {
  const dim3 blk(32, 8);
  k_adj_corner<T><<<dim3((a.g.N1 + 1 + 31) / 32, (a.g.N2 + 1 + 7) / 8), blk, 0, st>>>(a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_seed_impl(const Geom<T>& g, const T* U, T* lam, const int* gi, const int* gj,
                                 const double* target, int n, double* loss, cudaStream_t st) {
  k_adj_seed<T><<<1, 32, 0, st>>>(g, U, lam, gi, gj, target, n, loss);
  return cudaGetLastError();
}

}  // namespace vf
