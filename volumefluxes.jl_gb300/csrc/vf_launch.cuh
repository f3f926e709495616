// vf_launch.cuh -- host-side launchers of the step kernels, one set per real
// type. The Float64 set lives in vf_f64.cu (built with -fmad=false so every
// expression rounds as in Julia), the Float32 set in vf_f32.cu.
#pragma once
#include "vf_adjoint.cuh"
#include "vf_ensemble.cuh"
#include "vf_march.cuh"

// Float64 step kernels with faithful quotients and multiply-add contraction
// (vf_f64f.cu, a unit whose kernels live in their own namespace). `args` points
// to a vf::StepArgs<double>; same contract as vf::launch_step / launch_flux /
// launch_stage.
cudaError_t vf_faithful_launch_step(const void* args, const double* Uin, double* Uout, int parity, cudaStream_t st);
cudaError_t vf_faithful_launch_flux(const void* args, const double* Uin, int parity, cudaStream_t st);
cudaError_t vf_faithful_launch_stage(const void* args, const double* Uin, double* Uout, int parity, cudaStream_t st);
cudaError_t vf_faithful_configure();

namespace vf {

template <typename T>
struct StepArgs {
  Geom<T> g;
  Phys<T> p;
  int rk2;
  int variant;  // 0: column-marching kernels, 1: shared-memory tile kernels
  const T* B;
  T* L;
  T* S;
  StepRecord* rec;
  TmaMaps tma;  // Float64 tile kernels: TMA staging when tma.ok and the buffers match
  int arith;    // Float64 per-step kernels: 0 rounded as the reference, 1 faithful quotients (vf_f64f.cu)
};

// One full step reading Uin, writing Uout; parity selects the record slot.
cudaError_t launch_step(const StepArgs<double>& a, const double* Uin, double* Uout, int parity, cudaStream_t st);
cudaError_t launch_step(const StepArgs<float>& a, const float* Uin, float* Uout, int parity, cudaStream_t st);
// The two kernels of a step, separately (for per-kernel timing).
cudaError_t launch_flux(const StepArgs<double>& a, const double* Uin, int parity, cudaStream_t st);
cudaError_t launch_flux(const StepArgs<float>& a, const float* Uin, int parity, cudaStream_t st);
cudaError_t launch_stage(const StepArgs<double>& a, const double* Uin, double* Uout, int parity, cudaStream_t st);
cudaError_t launch_stage(const StepArgs<float>& a, const float* Uin, float* Uout, int parity, cudaStream_t st);
// Wall boundary update of a whole volume.
cudaError_t launch_bc(const Geom<double>& g, double* U, cudaStream_t st);
cudaError_t launch_bc(const Geom<float>& g, float* U, cudaStream_t st);
// Interior water volume into *out_dev (device double).
cudaError_t launch_volume(const Geom<double>& g, const double* U, const double* B, double* partial, int nblocks,
                          double* out_dev, cudaStream_t st);
cudaError_t launch_volume(const Geom<float>& g, const float* U, const float* B, double* partial, int nblocks,
                          double* out_dev, cudaStream_t st);
// Ensemble launch: n scenarios (items[order[i]]), one cluster of csize CTAs
// each; variant 0 column marching (Float32 only), 1 tiles.
cudaError_t launch_ensemble(const EnsItem<double>* items, const int* order, int n, int csize, int variant,
                            unsigned long long time_limit_ns, cudaStream_t st);
cudaError_t launch_ensemble(const EnsItem<float>* items, const int* order, int n, int csize, int variant,
                            unsigned long long time_limit_ns, cudaStream_t st);
// Clusters of csize CTAs that fit on the device at once (0: csize not launchable).
cudaError_t ensemble_max_clusters_f64(int csize, int variant, int* out);
cudaError_t ensemble_max_clusters_f32(int csize, int variant, int* out);
// Gather n interior cells' (w, hu, hv) into out (3 x n).
cudaError_t launch_sample(const Geom<double>& g, const double* U, const int* ij, int n, double* out, cudaStream_t st);
cudaError_t launch_sample(const Geom<float>& g, const float* U, const int* ij, int n, float* out, cudaStream_t st);
// Adjoint kernels (vf_adjoint.cuh), one launch each; *nblocks_out receives the
// number of dLoss/dCz partials k_adj_point wrote.
cudaError_t launch_adj_point(const AdjArgs<double>& a, int* nblocks_out, cudaStream_t st);
cudaError_t launch_adj_point(const AdjArgs<float>& a, int* nblocks_out, cudaStream_t st);
cudaError_t launch_adj_recon(const AdjArgs<double>& a, int dir, cudaStream_t st);
cudaError_t launch_adj_recon(const AdjArgs<float>& a, int dir, cudaStream_t st);
cudaError_t launch_adj_gather(const AdjArgs<double>& a, cudaStream_t st);
cudaError_t launch_adj_gather(const AdjArgs<float>& a, cudaStream_t st);
cudaError_t launch_adj_corner(const AdjArgs<double>& a, cudaStream_t st);
cudaError_t launch_adj_corner(const AdjArgs<float>& a, cudaStream_t st);
cudaError_t launch_adj_seed(const Geom<double>& g, const double* U, double* lam, const int* gi, const int* gj,
                            const double* target, int n, double* loss, cudaStream_t st);
cudaError_t launch_adj_seed(const Geom<float>& g, const float* U, float* lam, const int* gi, const int* gj,
                            const double* target, int n, double* loss, cudaStream_t st);
cudaError_t launch_adj_sum(const double* part, int n, double* acc, cudaStream_t st);
// Float64 quotients a[i] / b[i] as the Float64 kernels compute them (self-test).
cudaError_t launch_selftest_quotients(const double* a, const double* b, int n, double* q, cudaStream_t st);
cudaError_t launch_selftest_near_dry(const float* a, const float* b, int n, float* q, float* q64, cudaStream_t st);
// Opt the big-shared-memory kernels in on the current device (idempotent).
cudaError_t configure_kernels_f64();
cudaError_t configure_kernels_f32();

}  // namespace vf
