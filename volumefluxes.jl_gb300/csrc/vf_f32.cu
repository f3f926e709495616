// vf_f32.cu -- Float32 step kernels (multiply-add contraction and fast
// division allowed; the error is stated against the Float64 oracle).
#include "vf_step_impl.cuh"

namespace vf {
cudaError_t launch_step(const StepArgs<float>& a, const float* Uin, float* Uout, int parity, cudaStream_t st) {
  return launch_step_impl<float>(a, Uin, Uout, parity, st);
}
cudaError_t launch_flux(const StepArgs<float>& a, const float* Uin, int parity, cudaStream_t st) {
  return launch_flux_impl<float>(a, Uin, parity, st);
}
cudaError_t launch_stage(const StepArgs<float>& a, const float* Uin, float* Uout, int parity, cudaStream_t st) {
  return launch_stage_impl<float>(a, Uin, Uout, parity, st);
}
cudaError_t launch_bc(const Geom<float>& g, float* U, cudaStream_t st) { return launch_bc_impl<float>(g, U, st); }
cudaError_t launch_volume(const Geom<float>& g, const float* U, const float* B, double* partial, int nblocks,
                          double* out, cudaStream_t st) {
  return launch_volume_impl<float>(g, U, B, partial, nblocks, out, st);
}
cudaError_t launch_ensemble(const EnsItem<float>* items, const int* order, int n, int csize, int variant,
                            unsigned long long time_limit_ns, cudaStream_t st) {
  return launch_ensemble_impl<float>(items, order, n, csize, variant, time_limit_ns, st);
}
cudaError_t ensemble_max_clusters_f32(int csize, int variant, int* out) {
  return ensemble_max_clusters_impl<float>(csize, variant, out);
}
cudaError_t launch_adj_point(const AdjArgs<float>& a, int* nblocks_out, cudaStream_t st) {
  return launch_adj_point_impl<float>(a, nblocks_out, st);
}
cudaError_t launch_adj_recon(const AdjArgs<float>& a, int dir, cudaStream_t st) {
  return launch_adj_recon_impl<float>(a, dir, st);
}
cudaError_t launch_adj_gather(const AdjArgs<float>& a, cudaStream_t st) { return launch_adj_gather_impl<float>(a, st); }
cudaError_t launch_adj_corner(const AdjArgs<float>& a, cudaStream_t st) { return launch_adj_corner_impl<float>(a, st); }
cudaError_t launch_adj_seed(const Geom<float>& g, const float* U, float* lam, const int* gi, const int* gj,
                            const double* target, int n, double* loss, cudaStream_t st) {
  return launch_adj_seed_impl<float>(g, U, lam, gi, gj, target, n, loss, st);
}
cudaError_t launch_sample(const Geom<float>& g, const float* U, const int* ij, int n, float* out, cudaStream_t st) {
  k_sample<float><<<(n + 127) / 128, 128, 0, st>>>(g, U, ij, n, out);
  return cudaGetLastError();
}
// The near-dry velocity quotient as the Float32 kernels compute it (q) and the
// IEEE Float64 quotient rounded to Float32 (q64), element by element: the
// self-test of vf_selftest_near_dry_quotients.
static __global__ void k_selftest_near_dry(const float* a, const float* b, int n, float* q, float* q64) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    q[i] = f64_quotient_f32(a[i], b[i]);
    q64[i] = (float)((double)a[i] / (double)b[i]);
  }
}
cudaError_t launch_selftest_near_dry(const float* a, const float* b, int n, float* q, float* q64, cudaStream_t st) {
  k_selftest_near_dry<<<(n + 255) / 256, 256, 0, st>>>(a, b, n, q, q64);
  return cudaGetLastError();
}
cudaError_t configure_kernels_f32() { return configure_impl<float>(); }
}  // namespace vf
