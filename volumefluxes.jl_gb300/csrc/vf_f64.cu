// vf_f64.cu -- Float64 step kernels. Built with -fmad=false: no multiply-add
// contraction, IEEE division and square root, so each operation rounds as the
// reference's Julia code does.
#include "vf_step_impl.cuh"

namespace vf {
// a.arith == 1 hands the step to the faithful-quotient kernels of vf_f64f.cu.
cudaError_t launch_step(const StepArgs<double>& a, const double* Uin, double* Uout, int parity, cudaStream_t st) {
  if (a.arith == 1) return vf_faithful_launch_step(&a, Uin, Uout, parity, st);
  return launch_step_impl<double>(a, Uin, Uout, parity, st);
}
cudaError_t launch_flux(const StepArgs<double>& a, const double* Uin, int parity, cudaStream_t st) {
  if (a.arith == 1) return vf_faithful_launch_flux(&a, Uin, parity, st);
  return launch_flux_impl<double>(a, Uin, parity, st);
}
cudaError_t launch_stage(const StepArgs<double>& a, const double* Uin, double* Uout, int parity, cudaStream_t st) {
  if (a.arith == 1) return vf_faithful_launch_stage(&a, Uin, Uout, parity, st);
  return launch_stage_impl<double>(a, Uin, Uout, parity, st);
}
cudaError_t launch_bc(const Geom<double>& g, double* U, cudaStream_t st) { return launch_bc_impl<double>(g, U, st); }
cudaError_t launch_volume(const Geom<double>& g, const double* U, const double* B, double* partial, int nblocks,
                          double* out, cudaStream_t st) {
  return launch_volume_impl<double>(g, U, B, partial, nblocks, out, st);
}
cudaError_t launch_ensemble(const EnsItem<double>* items, const int* order, int n, int csize, int variant,
                            unsigned long long time_limit_ns, cudaStream_t st) {
  return launch_ensemble_impl<double>(items, order, n, csize, variant, time_limit_ns, st);
}
cudaError_t ensemble_max_clusters_f64(int csize, int variant, int* out) {
  return ensemble_max_clusters_impl<double>(csize, variant, out);
}
cudaError_t launch_adj_point(const AdjArgs<double>& a, int* nblocks_out, cudaStream_t st) {
  return launch_adj_point_impl<double>(a, nblocks_out, st);
}
cudaError_t launch_adj_recon(const AdjArgs<double>& a, int dir, cudaStream_t st) {
  return launch_adj_recon_impl<double>(a, dir, st);
}
cudaError_t launch_adj_gather(const AdjArgs<double>& a, cudaStream_t st) { return launch_adj_gather_impl<double>(a, st); }
cudaError_t launch_adj_corner(const AdjArgs<double>& a, cudaStream_t st) { return launch_adj_corner_impl<double>(a, st); }
cudaError_t launch_adj_seed(const Geom<double>& g, const double* U, double* lam, const int* gi, const int* gj,
                            const double* target, int n, double* loss, cudaStream_t st) {
  return launch_adj_seed_impl<double>(g, U, lam, gi, gj, target, n, loss, st);
}
cudaError_t launch_adj_sum(const double* part, int n, double* acc, cudaStream_t st) {
  k_adj_sum<<<1, 32, 0, st>>>(part, n, acc);
  return cudaGetLastError();
}
cudaError_t launch_sample(const Geom<double>& g, const double* U, const int* ij, int n, double* out, cudaStream_t st) {
  k_sample<double><<<(n + 127) / 128, 128, 0, st>>>(g, U, ij, n, out);
  return cudaGetLastError();
}
// The Float64 quotient of every kernel of this unit (a / b through Arith<double>::recip
// and div_by), element by element: the self-test of vf_selftest_quotients.
static __global__ void k_selftest_quotients(const double* a, const double* b, int n, double* q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) q[i] = Arith<double>::div_by(Arith<double>::recip(b[i]), a[i]);
}
cudaError_t launch_selftest_quotients(const double* a, const double* b, int n, double* q, cudaStream_t st) {
  k_selftest_quotients<<<(n + 255) / 256, 256, 0, st>>>(a, b, n, q);
  return cudaGetLastError();
}

cudaError_t configure_kernels_f64() {
  const cudaError_t e = configure_impl<double>();
  return e != cudaSuccess ? e : vf_faithful_configure();
}
}  // namespace vf
