// vf_f64f.cu -- Float64 per-step kernels held to a tolerance instead of to the
// reference's bits: quotients are faithful (about one ulp: a refined hardware
// reciprocal, one residual correction, products where several quotients share
// a divisor), cube roots come from the CUDA math library, and the unit is
// built with multiply-add contraction. Every other operation, the order of the
// passes and every branch are the bitwise kernels' own (the same source).
//
// The kernels are instantiated from the same headers as vf_f64.cu, so they
// are renamed into their own namespace (vf_faithful): two units must not hold
// different bodies under one kernel name. The argument block has the same
// layout in both namespaces (one header text, VF_FP64_FAITHFUL changes
// arithmetic only, no type).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#define VF_FP64_FAITHFUL 1
#define vf vf_faithful
#include "vf_step_impl.cuh"
#undef vf

namespace {
const vf_faithful::StepArgs<double>& args_of(const void* a) {
  return *static_cast<const vf_faithful::StepArgs<double>*>(a);
}
}  // namespace

cudaError_t vf_faithful_launch_step(const void* a, const double* Uin, double* Uout, int parity, cudaStream_t st) {
  return vf_faithful::launch_step_impl<double>(args_of(a), Uin, Uout, parity, st);
}
cudaError_t vf_faithful_launch_flux(const void* a, const double* Uin, int parity, cudaStream_t st) {
  return vf_faithful::launch_flux_impl<double>(args_of(a), Uin, parity, st);
}
cudaError_t vf_faithful_launch_stage(const void* a, const double* Uin, double* Uout, int parity, cudaStream_t st) {
  return vf_faithful::launch_stage_impl<double>(args_of(a), Uin, Uout, parity, st);
}
cudaError_t vf_faithful_configure() {
  using namespace vf_faithful;
  cudaError_t e = cudaFuncSetAttribute(k_flux<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(SmemFlux<double>));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_stage2<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(SmemStage<double>));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_flux_tma<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(SmemFlux<double>));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_stage2_tma<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(SmemStage<double>));
  return e;
}
