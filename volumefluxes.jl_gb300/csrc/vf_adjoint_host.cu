// vf_adjoint_host.cu -- the reverse sweep (vf_adjoint_*) of include/volumefluxes_sm103.h.
//
// Differentiates a loss of the state after N steps -- the gauge loss
// sum_g (w_g - target_g)^2 -- with respect to the bottom corners B and the
// friction coefficient Cz, with the dt sequence frozen from the forward pass.
// Memory follows sqrt(N) checkpointing: the forward pass keeps every K-th
// state (K ~ sqrt(N)); the reverse sweep walks the segments backwards,
// recomputes each segment's K states from its checkpoint, and reverses its
// steps one by one. A step is reversed from recomputed stage data (L(U^n),
// U1, L(U1)) by the adjoint kernels of vf_adjoint.cuh, stage 2 then stage 1.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "vf_handle.h"

struct vf_adjoint {
  vf_handle* h = nullptr;
  int n_steps = 0, K = 0, nseg = 0;
  size_t state_bytes = 0, plane_bytes = 0;
  void* init = nullptr;    // U^0 (with ghosts)
  void* ckpt = nullptr;    // nseg states
  void* seg = nullptr;     // K states of the segment being reversed
  void* U1 = nullptr;
  void* L0 = nullptr;
  void* L1 = nullptr;
  void* S0 = nullptr;
  void* S1 = nullptr;
  void* lam = nullptr;     // lambda of U^n (3 planes)
  void* lamU1 = nullptr;
  void* lamL = nullptr;
  void* lam_direct = nullptr;
  void* lam_base = nullptr;
  void* gBc = nullptr;
  void* C[2] = {nullptr, nullptr};    // 9 planes each
  void* gBf[2] = {nullptr, nullptr};  // 2 planes each
  double* gB = nullptr;    // (N1+1) x (N2+1)
  double* gCz_part = nullptr;
  double* gCz = nullptr;
  double* loss = nullptr;
  int* gauges = nullptr;
  double* target = nullptr;
  int gauge_cap = 0;
  vf::StepRecord* rec = nullptr;
  vf::StepRecord rec_h;
  std::vector<double> dts;
  std::vector<double> ts;  // start time of every step of the forward pass (time-dependent sources)
  bool have_forward = false;
  std::string err;
};

namespace {

thread_local std::string g_adj_error;

int afail(vf_adjoint* a, int code, const std::string& msg) {
  if (a) a->err = msg;
  else g_adj_error = msg;
  return code;
}

#define VF_ACK(a, call)                                                              \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) return afail((a), VF_ECUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

void* off(void* base, size_t bytes) { return static_cast<char*>(base) + bytes; }

void free_all(vf_adjoint* a) {
  cudaStream_t st = a->h ? a->h->stream : nullptr;
  void* ps[] = {a->init, a->ckpt, a->seg, a->U1, a->L0, a->L1, a->S0, a->S1, a->lam, a->lamU1, a->lamL,
                a->lam_direct, a->lam_base, a->gBc, a->C[0], a->C[1], a->gBf[0], a->gBf[1], a->gB,
                a->gCz_part, a->gCz, a->loss, a->gauges, a->target, a->rec};
  for (void* p : ps)
    if (p) cudaFreeAsync(p, st);
  if (st) cudaStreamSynchronize(st);
}

bool alloc(vf_adjoint* a, void** p, size_t bytes) {
  cudaMemPool_t pool = vf::device_pool(a->h->device);
  if (!pool || cudaMallocFromPoolAsync(p, bytes, pool, a->h->stream) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return false;
  }
  return cudaMemsetAsync(*p, 0, bytes, a->h->stream) == cudaSuccess;
}

template <typename T>
vf::StepArgs<T>& args_of(vf_handle* h);
template <>
vf::StepArgs<double>& args_of<double>(vf_handle* h) { return h->ad; }
template <>
vf::StepArgs<float>& args_of<float>(vf_handle* h) { return h->af; }

int set_dt(vf_adjoint* a, double dt, double t) {
  std::memset(&a->rec_h, 0, sizeof(a->rec_h));
  a->rec_h.active[0] = 1;
  a->rec_h.t[0] = t;
  a->rec_h.explicit_mode = 1;
  a->rec_h.force_dt = 1;
  a->rec_h.forced_dt = dt;
  VF_ACK(a, cudaMemcpyAsync(a->rec, &a->rec_h, sizeof(vf::StepRecord), cudaMemcpyHostToDevice, a->h->stream));
  // the record is pageable host memory: let the copy finish before it changes
  VF_ACK(a, cudaStreamSynchronize(a->h->stream));
  return VF_OK;
}

// One forward step of the checkpointed recomputation: Uin -> Uout with dt.
template <typename T>
int fwd_step(vf_adjoint* a, const void* Uin, void* Uout, double dt, double t) {
  vf_handle* h = a->h;
  if (int rc = set_dt(a, dt, t)) return rc;
  vf::StepArgs<T> s = args_of<T>(h);
  s.L = static_cast<T*>(a->L0);
  s.S = static_cast<T*>(a->S0);
  s.rec = a->rec;
  s.arith = VF_ARITH_REFERENCE;  // the reverse sweep differentiates the reference-rounded step
  VF_ACK(a, vf::launch_step(s, static_cast<const T*>(Uin), static_cast<T*>(Uout), 0, h->stream));
  h->launches += 2;
  return VF_OK;
}

template <typename T>
vf::AdjArgs<T> adj_args(vf_adjoint* a, double dt) {
  vf_handle* h = a->h;
  const vf::StepArgs<T>& s = args_of<T>(h);
  vf::AdjArgs<T> x;
  std::memset(&x, 0, sizeof(x));
  x.g = s.g;
  x.p = s.p;
  x.B = s.B;
  x.dt = dt;
  x.lamL = static_cast<T*>(a->lamL);
  x.lam_direct = static_cast<T*>(a->lam_direct);
  x.lam_base = static_cast<T*>(a->lam_base);
  x.gBc = static_cast<T*>(a->gBc);
  x.gCz_part = a->gCz_part;
  x.C[0] = static_cast<T*>(a->C[0]);
  x.C[1] = static_cast<T*>(a->C[1]);
  x.gBf[0] = static_cast<T*>(a->gBf[0]);
  x.gBf[1] = static_cast<T*>(a->gBf[1]);
  x.gB = a->gB;
  return x;
}

// One stage in reverse: pointwise part, both reconstructions, gather, corners.
template <typename T>
int reverse_stage(vf_adjoint* a, vf::AdjArgs<T> x) {
  cudaStream_t st = a->h->stream;
  int nb = 0;
  VF_ACK(a, vf::launch_adj_point(x, &nb, st));
  VF_ACK(a, vf::launch_adj_sum(a->gCz_part, nb, a->gCz, st));
  VF_ACK(a, vf::launch_adj_recon(x, 0, st));
  VF_ACK(a, vf::launch_adj_recon(x, 1, st));
  VF_ACK(a, vf::launch_adj_gather(x, st));
  VF_ACK(a, vf::launch_adj_corner(x, st));
  a->h->launches += 6;
  return VF_OK;
}

// Reverse of step n whose input state is U0 (start time t): lam holds lambda of
// U^{n+1} on entry and lambda of U^n on return. Forward Euler is the RK2 first
// stage alone (src/timestepper/forwardeuler.jl:28-47): its output is U^{n+1}.
template <typename T>
int reverse_step(vf_adjoint* a, const void* U0, double dt, double t) {
  vf_handle* h = a->h;
  if (int rc = set_dt(a, dt, t)) return rc;
  vf::StepArgs<T> s = args_of<T>(h);
  s.rec = a->rec;
  s.arith = VF_ARITH_REFERENCE;
  // recompute L(U0), S(U0) (and for RK2 U1, L(U1), S(U1))
  s.L = static_cast<T*>(a->L0);
  s.S = static_cast<T*>(a->S0);
  VF_ACK(a, vf::launch_flux(s, static_cast<const T*>(U0), 0, h->stream));
  h->launches += 1;
  if (!s.rk2) {
    vf::AdjArgs<T> x1 = adj_args<T>(a, dt);
    x1.stage2 = 0;
    x1.Uprev = static_cast<const T*>(U0);
    x1.L = static_cast<const T*>(a->L0);
    x1.lam_out = static_cast<const T*>(a->lam);
    x1.lam_in = static_cast<T*>(a->lamU1);
    if (int rc = reverse_stage<T>(a, x1)) return rc;
    std::swap(a->lam, a->lamU1);  // lambda of U^n now in lam
    return VF_OK;
  }
  vf::StepArgs<T> fe = s;
  fe.rk2 = 0;
  VF_ACK(a, vf::launch_stage(fe, static_cast<const T*>(U0), static_cast<T*>(a->U1), 0, h->stream));
  s.L = static_cast<T*>(a->L1);
  s.S = static_cast<T*>(a->S1);
  VF_ACK(a, vf::launch_flux(s, static_cast<const T*>(a->U1), 0, h->stream));
  h->launches += 2;
  // stage 2
  vf::AdjArgs<T> x2 = adj_args<T>(a, dt);
  x2.stage2 = 1;
  x2.Uprev = static_cast<const T*>(a->U1);
  x2.Ubase = static_cast<const T*>(U0);
  x2.L = static_cast<const T*>(a->L1);
  x2.lam_out = static_cast<const T*>(a->lam);
  x2.lam_in = static_cast<T*>(a->lamU1);
  if (int rc = reverse_stage<T>(a, x2)) return rc;
  // stage 1
  vf::AdjArgs<T> x1 = adj_args<T>(a, dt);
  x1.stage2 = 0;
  x1.Uprev = static_cast<const T*>(U0);
  x1.L = static_cast<const T*>(a->L0);
  x1.lam_out = static_cast<const T*>(a->lamU1);
  x1.lam_in = static_cast<T*>(a->lam);
  return reverse_stage<T>(a, x1);
}

template <typename T>
int backward_impl(vf_adjoint* a, const int32_t* gi, const int32_t* gj, const double* target, int32_t n_g,
                  double* loss_out, double* grad_B, double* grad_Cz) {
  vf_handle* h = a->h;
  cudaStream_t st = h->stream;
  const vf::Geom<T>& g = args_of<T>(h).g;
  if (n_g > a->gauge_cap) {
    if (a->gauges) cudaFreeAsync(a->gauges, st);
    if (a->target) cudaFreeAsync(a->target, st);
    a->gauges = nullptr;
    a->target = nullptr;
    if (!alloc(a, reinterpret_cast<void**>(&a->gauges), sizeof(int) * 2 * (size_t)n_g) ||
        !alloc(a, reinterpret_cast<void**>(&a->target), sizeof(double) * (size_t)n_g))
      return afail(a, VF_ENOMEM, "gauge buffers");
    a->gauge_cap = n_g;
  }
  std::vector<int> gg(2 * (size_t)n_g);
  for (int k = 0; k < n_g; ++k) {
    if (gi[k] < 0 || gj[k] < 0 || gi[k] >= g.nx || gj[k] >= g.ny) return afail(a, VF_EINVAL, "gauge outside the grid");
    gg[k] = gi[k];
    gg[n_g + k] = gj[k];
  }
  VF_ACK(a, cudaMemcpyAsync(a->gauges, gg.data(), sizeof(int) * gg.size(), cudaMemcpyHostToDevice, st));
  VF_ACK(a, cudaMemcpyAsync(a->target, target, sizeof(double) * (size_t)n_g, cudaMemcpyHostToDevice, st));
  VF_ACK(a, cudaMemsetAsync(a->lam, 0, a->state_bytes, st));
  VF_ACK(a, cudaMemsetAsync(a->gB, 0, sizeof(double) * (size_t)(g.N1 + 1) * (g.N2 + 1), st));
  VF_ACK(a, cudaMemsetAsync(a->gCz, 0, sizeof(double), st));
  VF_ACK(a, vf::launch_adj_seed(g, static_cast<const T*>(h->U[0]), static_cast<T*>(a->lam), a->gauges,
                                a->gauges + n_g, a->target, n_g, a->loss, st));
  VF_ACK(a, cudaStreamSynchronize(st));  // the host vectors above go out of scope
  for (int s = a->nseg - 1; s >= 0; --s) {
    const int start = s * a->K;
    const int end = std::min(a->n_steps, start + a->K);
    VF_ACK(a, cudaMemcpyAsync(a->seg, off(a->ckpt, (size_t)s * a->state_bytes), a->state_bytes,
                              cudaMemcpyDeviceToDevice, st));
    for (int n = start; n + 1 < end; ++n)
      if (int rc = fwd_step<T>(a, off(a->seg, (size_t)(n - start) * a->state_bytes),
                               off(a->seg, (size_t)(n - start + 1) * a->state_bytes), a->dts[n], a->ts[n]))
        return rc;
    for (int n = end - 1; n >= start; --n)
      if (int rc = reverse_step<T>(a, off(a->seg, (size_t)(n - start) * a->state_bytes), a->dts[n], a->ts[n]))
        return rc;
  }
  double gcz = 0, loss = 0;
  VF_ACK(a, cudaMemcpyAsync(&gcz, a->gCz, sizeof(double), cudaMemcpyDeviceToHost, st));
  VF_ACK(a, cudaMemcpyAsync(&loss, a->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
  if (grad_B)
    VF_ACK(a, cudaMemcpyAsync(grad_B, a->gB, sizeof(double) * (size_t)(g.N1 + 1) * (g.N2 + 1),
                              cudaMemcpyDeviceToHost, st));
  VF_ACK(a, cudaStreamSynchronize(st));
  if (grad_Cz) *grad_Cz = gcz;
  if (loss_out) *loss_out = loss;
  return VF_OK;
}

}  // namespace

extern "C" {

int vf_adjoint_create(vf_handle* h, int32_t n_steps, int32_t checkpoint_every, vf_adjoint** out) {
  if (!out) return afail(nullptr, VF_EINVAL, "out is NULL");
  *out = nullptr;
  if (!h || n_steps < 1) return afail(nullptr, VF_EINVAL, "need a handle and n_steps >= 1");
  if (int rc = vf::handle_ready(h)) return afail(nullptr, rc, std::string("handle not ready: ") + h->err);
  const vf_config& c = h->cfg;
  if ((c.stepper != VF_STEPPER_RK2 && c.stepper != VF_STEPPER_FE) ||
      (c.reconstruction != VF_REC_LINEAR && c.reconstruction != VF_REC_NONE) ||
      (c.bc != VF_BC_WALL && c.bc != VF_BC_PERIODIC) || c.bottom_is_constant)
    return afail(nullptr, VF_EINVAL,
                 "the adjoint covers RungeKutta2 and ForwardEulerStepper, LinearReconstruction and NoReconstruction, "
                 "WallBC and PeriodicBC, and a BottomTopography2D");
  if (c.friction != VF_FRICTION_NONE && c.friction != VF_FRICTION_BSA2012 && c.friction != VF_FRICTION_FCG2016 &&
      c.friction != VF_FRICTION_BH2021)
    return afail(nullptr, VF_EINVAL, "unknown friction law");
  for (int i = 0; i < c.n_sources; ++i)
    if (c.source_kind[i] != VF_SRC_BOTTOM && c.source_kind[i] != VF_SRC_CONST_RAIN &&
        c.source_kind[i] != VF_SRC_CONST_INFIL && c.source_kind[i] != VF_SRC_TIME_RAIN &&
        c.source_kind[i] != VF_SRC_HORTON)
      return afail(nullptr, VF_EINVAL,
                   "the adjoint covers SourceTermBottom, ConstantRain, ConstantInfiltration, TimeDependentRain and "
                   "HortonInfiltration (a FunctionalRain field changes on the host between steps)");
  vf_adjoint* a = new (std::nothrow) vf_adjoint();
  if (!a) return afail(nullptr, VF_ENOMEM, "host allocation failed");
  a->h = h;
  a->n_steps = n_steps;
  a->K = checkpoint_every > 0 ? checkpoint_every : std::max(1, (int)std::lround(std::sqrt((double)n_steps)));
  a->nseg = (n_steps + a->K - 1) / a->K;
  a->plane_bytes = (size_t)h->PS * h->elem;
  a->state_bytes = 3 * a->plane_bytes;
  const size_t corners = (size_t)(h->N1 + 1) * (h->N2 + 1);
  bool ok = alloc(a, &a->init, a->state_bytes) && alloc(a, &a->ckpt, a->state_bytes * a->nseg) &&
            alloc(a, &a->seg, a->state_bytes * a->K) && alloc(a, &a->U1, a->state_bytes) &&
            alloc(a, &a->L0, a->state_bytes) && alloc(a, &a->L1, a->state_bytes) &&
            alloc(a, &a->S0, a->plane_bytes) && alloc(a, &a->S1, a->plane_bytes) &&
            alloc(a, &a->lam, a->state_bytes) && alloc(a, &a->lamU1, a->state_bytes) &&
            alloc(a, &a->lamL, a->state_bytes) && alloc(a, &a->lam_direct, a->state_bytes) &&
            alloc(a, &a->lam_base, a->state_bytes) && alloc(a, &a->gBc, a->plane_bytes) &&
            alloc(a, &a->C[0], 9 * a->plane_bytes) && alloc(a, &a->C[1], 9 * a->plane_bytes) &&
            alloc(a, &a->gBf[0], 2 * a->plane_bytes) && alloc(a, &a->gBf[1], 2 * a->plane_bytes) &&
            alloc(a, reinterpret_cast<void**>(&a->gB), sizeof(double) * corners) &&
            alloc(a, reinterpret_cast<void**>(&a->gCz_part), sizeof(double) * (size_t)((h->cfg.nx + 31) / 32) *
                                                                 ((h->cfg.ny + 7) / 8)) &&
            alloc(a, reinterpret_cast<void**>(&a->gCz), sizeof(double)) &&
            alloc(a, reinterpret_cast<void**>(&a->loss), sizeof(double)) &&
            alloc(a, reinterpret_cast<void**>(&a->rec), sizeof(vf::StepRecord));
  ok = ok && cudaMemcpyAsync(a->init, h->U[0], a->state_bytes, cudaMemcpyDeviceToDevice, h->stream) == cudaSuccess;
  ok = ok && cudaStreamSynchronize(h->stream) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    free_all(a);
    delete a;
    return afail(nullptr, VF_ENOMEM, "adjoint buffers could not be allocated");
  }
  *out = a;
  return VF_OK;
}

int vf_adjoint_forward(vf_adjoint* a, const double* frozen_dts, double* dts_out) {
  if (!a) return afail(nullptr, VF_EINVAL, "NULL adjoint");
  vf_handle* h = a->h;
  VF_ACK(a, cudaSetDevice(h->device));
  VF_ACK(a, cudaMemcpyAsync(h->U[0], a->init, a->state_bytes, cudaMemcpyDeviceToDevice, h->stream));
  a->dts.assign(a->n_steps, 0.0);
  a->ts.assign(a->n_steps, 0.0);
  double t = 0.0;
  for (int n = 0; n < a->n_steps; ++n) {
    a->ts[n] = t;
    if (n % a->K == 0)
      VF_ACK(a, cudaMemcpyAsync(off(a->ckpt, (size_t)(n / a->K) * a->state_bytes), h->U[0], a->state_bytes,
                                cudaMemcpyDeviceToDevice, h->stream));
    int rc;
    double dt = 0;
    if (frozen_dts) {
      dt = frozen_dts[n];
      rc = vf_step_fixed(h, dt, t);
    } else {
      rc = vf_step(h, INFINITY, t, &dt);
    }
    if (rc) return afail(a, rc, std::string("forward step: ") + h->err);
    a->dts[n] = dt;
    t += dt;
  }
  if (dts_out) std::memcpy(dts_out, a->dts.data(), sizeof(double) * a->n_steps);
  a->have_forward = true;
  return VF_OK;
}

int vf_adjoint_backward(vf_adjoint* a, const int32_t* gauge_i, const int32_t* gauge_j, const double* target,
                        int32_t n_gauges, double* loss_out, double* grad_B, double* grad_Cz) {
  if (!a) return afail(nullptr, VF_EINVAL, "NULL adjoint");
  if (!a->have_forward) return afail(a, VF_ESTATE, "run vf_adjoint_forward first");
  if (n_gauges < 1 || !gauge_i || !gauge_j || !target) return afail(a, VF_EINVAL, "need gauges and targets");
  VF_ACK(a, cudaSetDevice(a->h->device));
  return a->h->elem == 8 ? backward_impl<double>(a, gauge_i, gauge_j, target, n_gauges, loss_out, grad_B, grad_Cz)
                         : backward_impl<float>(a, gauge_i, gauge_j, target, n_gauges, loss_out, grad_B, grad_Cz);
}

void vf_adjoint_destroy(vf_adjoint* a) {
  if (!a) return;
  cudaSetDevice(a->h->device);
  free_all(a);
  delete a;
}

const char* vf_adjoint_last_error(vf_adjoint* a) { return a ? a->err.c_str() : g_adj_error.c_str(); }

}  // extern "C"
