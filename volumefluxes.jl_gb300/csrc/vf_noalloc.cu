// vf_noalloc.cu -- water volume of a caller-owned device state, with no
// device allocation at all.
//
// vf_water_volume() sums through scratch buffers that vf_create() allocated.
// Some callers cannot let a library call cudaMalloc: code whose device memory
// is owned by another allocator that must account for every byte (CUDA.jl's
// pool, a framework's caching allocator), or loops that cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree may imply. For them this
// entry point reads a state they allocated, writes the result to a device
// double they allocated, and keeps its own scratch -- one Float64 partial sum
// per interior row -- in a fixed file-scope device array.
//
// Limits and sharing rules:
//  - at most VF_STATIC_MAX_ROWS interior rows (ny); larger grids are rejected;
//  - the array is loaded with the library and held on every GPU that uses it
//    until the process exits;
//  - every call on a device uses the same array: calls whose kernels overlap
//    on the GPU (different streams, no ordering between them) race;
//  - a call made outside stream capture looks the array's address up with the
//    device current (the address can change when the device or its primary
//    context is reset, e.g. cudaDeviceReset or CUDA.jl's device_reset!, which
//    reloads the module); a call made during capture uses the address the
//    last uncaptured call on that device found. So make one call on a device
//    before capturing, and again after any reset of it.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/volumefluxes_sm103.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

// Per-row partial sums. Every call overwrites rows [0, ny) before the final
// pass reads them, so nothing has to be cleared between calls.
static __device__ __align__(256) double g_row_sums[VF_STATIC_MAX_ROWS];

std::mutex g_mu;
double* g_row_sums_addr[kMaxDevices] = {};

__device__ __forceinline__ double reduce_block(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  return red[0];
}

// One block per interior row: sum over the row of (w - B_cell) * dx * dy in a
// fixed order. The dense layout is the reference's Volume: plane stride
// N1*N2, row stride N1 (x fastest); corners (N1+1) x (N2+1).
template <typename T>
__global__ void k_row_volume(const T* __restrict__ state, const T* __restrict__ B, int nx, int gc, int N1,
                             double dx, double dy, int bconst, double bval, double* row_sums) {
  __shared__ double red[kThreads];
  const int j = gc + blockIdx.x;
  double acc = 0.0;
  for (int i = gc + threadIdx.x; i < gc + nx; i += kThreads) {
    double Bc = (double)(T)bval;  // the constant bottom in the state's type, as vf_water_volume holds it
    if (!bconst) {
      const long long b = (long long)j * (N1 + 1) + i;
      const long long W = N1 + 1;
      Bc = (double)((T)0.25 * (((B[b] + B[b + 1]) + B[b + W]) + B[b + W + 1]));
    }
    acc += ((double)state[(long long)j * N1 + i] - Bc) * dx * dy;
  }
  const double s = reduce_block(acc, red);
  if (threadIdx.x == 0) row_sums[blockIdx.x] = s;
}

__global__ void k_sum_rows(const double* __restrict__ row_sums, int ny, double* out) {
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (int j = threadIdx.x; j < ny; j += kThreads) acc += row_sums[j];
  const double s = reduce_block(acc, red);
  if (threadIdx.x == 0) *out = s;
}

// Address of g_row_sums on the current device. Outside stream capture it is
// looked up afresh (cheap, and right after a device reset); during capture the
// last address found on this device is used, since the lookup may load the
// module, which capture does not allow.
int row_sums_address(cudaStream_t st, double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return VF_ECUDA;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  const bool capturing = cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!capturing) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_row_sums) != cudaSuccess || !p) return VF_ECUDA;
    g_row_sums_addr[dev] = static_cast<double*>(p);
  }
  if (!g_row_sums_addr[dev]) return VF_ECUDA;
  *out = g_row_sums_addr[dev];
  return VF_OK;
}

}  // namespace

namespace vf {
void set_global_error(const char* msg);  // vf_abi.cu: the message vf_last_error(NULL) returns
}

namespace {
int fail(int code, const char* msg) {
  vf::set_global_error(msg);
  return code;
}
}  // namespace

extern "C" int vf_water_volume_static(const void* state_dev, const void* B_dev, int32_t nx, int32_t ny, int32_t gc,
                                      int32_t real_bytes, double dx, double dy, int32_t bottom_is_constant,
                                      double bottom_constant, double* out_dev, void* stream) {
  if (!state_dev || !out_dev || (!bottom_is_constant && !B_dev)) return fail(VF_EINVAL, "NULL pointer argument");
  if (nx < 1 || ny < 1 || gc < 0) return fail(VF_EINVAL, "nx and ny must be positive, gc non-negative");
  if (ny > VF_STATIC_MAX_ROWS)
    return fail(VF_EINVAL, "ny exceeds the static scratch capacity of VF_STATIC_MAX_ROWS interior rows");
  if (real_bytes != 8 && real_bytes != 4) return fail(VF_EINVAL, "real_bytes must be 8 or 4");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* rows = nullptr;
  if (row_sums_address(st, &rows) != VF_OK)
    return fail(VF_ECUDA, "no address of the row-sum scratch on this device (make one call outside stream capture "
                          "first; cudaGetSymbolAddress failed or the stream is capturing)");
  const int N1 = nx + 2 * gc;
  if (real_bytes == 8) {
    k_row_volume<double><<<ny, kThreads, 0, st>>>(static_cast<const double*>(state_dev),
                                                  static_cast<const double*>(B_dev), nx, gc, N1, dx, dy,
                                                  bottom_is_constant, bottom_constant, rows);
  } else {
    k_row_volume<float><<<ny, kThreads, 0, st>>>(static_cast<const float*>(state_dev),
                                                 static_cast<const float*>(B_dev), nx, gc, N1, dx, dy,
                                                 bottom_is_constant, bottom_constant, rows);
  }
  k_sum_rows<<<1, kThreads, 0, st>>>(rows, ny, out_dev);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(VF_ECUDA, cudaGetErrorString(e));
  return VF_OK;
}
