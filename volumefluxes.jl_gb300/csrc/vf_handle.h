// vf_handle.h -- the handle behind the opaque vf_handle of the C ABI, shared
// by the units that implement the ABI (vf_abi.cu, vf_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/volumefluxes_sm103.h"
#include "vf_launch.cuh"

struct vf_handle {
  vf_config cfg;
  int device = 0;
  size_t elem = 8;
  cudaStream_t stream = nullptr;
  int N1 = 0, N2 = 0;
  long long P = 0, PS = 0, PB = 0;
  void* U[2] = {nullptr, nullptr};
  void* L = nullptr;
  void* S = nullptr;
  void* B = nullptr;
  vf::StepRecord* rec = nullptr;
  vf::StepRecord* rec_h = nullptr;  // host copy (pageable)
  double* partial = nullptr;
  double* vol_out = nullptr;
  void* src_field[VF_MAX_SOURCES] = {};   // per-cell source arrays (state layout)
  double* src_tab[VF_MAX_SOURCES] = {};   // breakpoints then rates/3600
  int src_tab_n[VF_MAX_SOURCES] = {};
  int vol_blocks = 0;
  vf::StepArgs<double> ad;
  vf::StepArgs<float> af;
  bool have_state = false;
  bool have_bottom = false;
  std::string err;
  long long launches = 0;
  int* sample_ij = nullptr;   // gauge indices and values of vf_sample_cells
  void* sample_out = nullptr;
  int sample_cap = 0;
  cudaGraphExec_t chunk_exec = nullptr;  // captured chunk of steps (wide batch members)
  int chunk_k = 0;                        // its step count; 0: recapture
  void* chunk_u0 = nullptr;               // U[0] when captured (the buffers swap between calls)
};

namespace vf {
// Checks that a handle can step (state, bottom, tables and fields uploaded)
// and makes its device current; on failure records the message on h.
int handle_ready(vf_handle* h);
// Device-resident time loop of vf_simulate, driven asynchronously: write the
// loop's record (t0, end time, match_endtime, maximum_timestep < 0: none) to
// the device on the handle's stream.
int handle_begin_loop(vf_handle* h, double t0, double endtime, int match_endtime, double maximum_timestep);
// Enqueue n steps with global indices first, first+1, ... on the handle's
// stream (a step whose record slot is inactive does nothing).
int handle_enqueue_steps(vf_handle* h, long long first, int n);
// Enqueue k steps (k even, first even) as one CUDA graph launch; the graph is
// captured on first use and kept with the handle.
int handle_enqueue_chunk(vf_handle* h, int k);
// Device bytes vf_create allocates for a configuration (validated or not).
size_t handle_device_bytes(const vf_config* c);
// Records a message for the create-time error slot (vf_last_error(NULL)).
void set_global_error(const char* msg);
// The library's stream-ordered device memory pool of a device (created on
// first use, memory kept for reuse). Allocating and freeing from it never
// synchronises the device, so handles can come and go while other work runs.
cudaMemPool_t device_pool(int device);
}  // namespace vf
