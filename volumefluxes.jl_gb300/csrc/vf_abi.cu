// vf_abi.cu -- the extern "C" boundary declared in include/volumefluxes_sm103.h.
//
// Owns device memory and the stream of each handle, converts between the
// reference's dense Volume layout and the padded device layout, and drives the
// step kernels (vf_launch.cuh). No CPU fallback exists: every compute entry
// point runs on the GPU or returns an error.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <new>
#include <string>

#include "vf_handle.h"

namespace {

thread_local std::string g_create_error;

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

}  // namespace

namespace vf {
void set_global_error(const char* msg) { g_create_error = msg; }

cudaMemPool_t device_pool(int device) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  if (device < 0 || device >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[device]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    unsigned long long keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[device] = pool;
  }
  return pools[device];
}
}  // namespace vf

namespace {

// Stream-ordered allocation from the library pool on the handle's stream.
bool dalloc(vf_handle* h, void** p, size_t bytes) {
  cudaMemPool_t pool = vf::device_pool(h->device);
  if (!pool) return false;
  if (cudaMallocFromPoolAsync(p, bytes, pool, h->stream) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return false;
  }
  return true;
}

void dfree(vf_handle* h, void* p) {
  if (p) cudaFreeAsync(p, h->stream);
}

int fail(vf_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  else g_create_error = msg;
  return code;
}

int cuda_fail(vf_handle* h, cudaError_t e, const char* what) {
  return fail(h, VF_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define VF_CK(h, call)                                          \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) return cuda_fail((h), e_, #call);    \
  } while (0)

template <typename T>
void fill_geom(const vf_handle* h, vf::Geom<T>& g) {
  g.nx = h->cfg.nx;
  g.ny = h->cfg.ny;
  g.gc = h->cfg.gc;
  g.N1 = h->N1;
  g.N2 = h->N2;
  g.P = h->P;
  g.PS = h->PS;
  g.PB = h->PB;
  g.bottom_const = h->cfg.bottom_is_constant;
  g.bconst = (T)h->cfg.bottom_constant;
  g.dx = (h->cfg.extent[1] - h->cfg.extent[0]) / h->cfg.nx;
  g.dy = (h->cfg.extent[3] - h->cfg.extent[2]) / h->cfg.ny;
  // Simulator.cfl is stored in the backend's real type (src/simulator.jl:68).
  g.cfl = (double)(T)h->cfg.cfl;
  g.bc = h->cfg.bc;
}

// Float32 velocities with |h| below this many desingularizing_kappa are
// divided in Float64.
constexpr double VF_NEAR_DRY_FACTOR = 2.0;

template <typename T>
void fill_phys(const vf_handle* h, vf::Phys<T>& p) {
  const vf_config& c = h->cfg;
  p.g = (T)c.g;
  p.neg_g = (T)(-c.g);
  p.rho = (T)c.rho;
  p.c2 = (T)((0.5 * c.rho) * c.g);
  p.cutoff = (T)c.depth_cutoff;
  p.kappa = (T)c.desingularizing_kappa;
  p.theta = (T)c.theta;
  const double dx = (c.extent[1] - c.extent[0]) / c.nx;
  const double dy = (c.extent[3] - c.extent[2]) / c.ny;
  p.inv_dx = (T)(1 / dx);
  p.inv_dy = (T)(1 / dy);
  p.dx = (T)dx;
  p.dy = (T)dy;
  int ex = 0;
  p.dx_pow2 = std::frexp(dx, &ex) == 0.5 ? 1 : 0;
  p.dy_pow2 = std::frexp(dy, &ex) == 0.5 ? 1 : 0;
  p.Cz = (T)c.friction_Cz;
  // Float32: velocities of cells and faces with |h| < VF_NEAR_DRY_FACTOR *
  // desingularizing_kappa (the depth scale of the desingularised division,
  // src/equations/equation.jl:40-67) are divided in Float64;
  // VF_F32_NEAR_DRY=0 turns it off, VF_F32_NEAR_DRY_FACTOR overrides the factor.
  const char* nd = std::getenv("VF_F32_NEAR_DRY");
  const char* nf = std::getenv("VF_F32_NEAR_DRY_FACTOR");
  const double factor = nf ? std::atof(nf) : VF_NEAR_DRY_FACTOR;
  p.near_dry = (sizeof(T) == 4 && !(nd && std::strcmp(nd, "0") == 0)) ? (T)(factor * c.desingularizing_kappa) : (T)0;
  p.friction = c.friction;
  p.n_bottom = 0;
  p.n_point = 0;
  p.rec_none = c.reconstruction == VF_REC_NONE ? 1 : 0;
  p.any_dynamic = 0;
  for (int i = 0; i < 8; ++i) {
    p.point_add[i] = (T)0;
    p.point_kind[i] = vf::kConstant;
    p.point_field[i] = nullptr;
    p.tab_t[i] = p.tab_r[i] = nullptr;
    p.tab_n[i] = 0;
    p.horton[i][0] = p.horton[i][1] = p.horton[i][2] = 0.0;
  }
  for (int i = 0; i < c.n_sources; ++i) {
    const int k = c.source_kind[i];
    if (k == VF_SRC_BOTTOM) {
      ++p.n_bottom;
      continue;
    }
    const int n = p.n_point++;
    if (k == VF_SRC_CONST_RAIN) {
      p.point_add[n] = (T)(c.source_rate[i] / 3600);  // compute_rain, source_term_rain.jl:30
    } else if (k == VF_SRC_CONST_INFIL) {
      p.point_add[n] = (T)(-c.source_rate[i]);        // x - r == x + (-r) exactly
    } else if (k == VF_SRC_TIME_RAIN) {
      p.point_kind[n] = vf::kTable;
      p.tab_n[n] = h->src_tab_n[i];
      p.tab_t[n] = h->src_tab[i];
      p.tab_r[n] = h->src_tab[i] ? h->src_tab[i] + h->src_tab_n[i] : nullptr;
      p.any_dynamic = 1;
    } else if (k == VF_SRC_HORTON) {
      p.point_kind[n] = vf::kHorton;
      p.point_field[n] = static_cast<const T*>(h->src_field[i]);
      p.horton[n][0] = c.source_rate[i];
      p.horton[n][1] = c.source_aux[i][0];
      p.horton[n][2] = c.source_aux[i][1];
      p.any_dynamic = 1;
    } else if (k == VF_SRC_RAIN_FIELD) {
      p.point_kind[n] = vf::kField;
      p.point_field[n] = static_cast<const T*>(h->src_field[i]);
      p.any_dynamic = 1;
    }
  }
  double sum = 0.0;
  for (int n = 0; n < p.n_point; ++n) sum += (double)p.point_add[n];
  p.point_sum = (T)sum;
  p.bottom_g = (T)(p.n_bottom * -c.g);
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (no link-time dependency on libcuda).
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// Tiled tensor map of a Float64 array of `planes` planes (planes > 1: 3D) with
// rows of `pitch` elements, plane stride `ps`, extent (nx, ny) elements; the
// box is (bx, by[, planes]). Out-of-range elements read as zero.
bool encode_f64(CUtensorMap* m, const void* base, long long nx, long long ny, long long pitch, long long ps,
                int planes, int bx, int by) {
  auto fn = encode_tiled();
  if (!fn || !base) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)planes};
  const cuuint64_t strides[2] = {(cuuint64_t)(pitch * 8), (cuuint64_t)(ps * 8)};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)planes};
  const cuuint32_t estr[3] = {1, 1, 1};
  const cuuint32_t rank = planes > 1 ? 3 : 2;
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, rank, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps of a Float64 handle's state, derivative, friction and corner
// buffers for the TMA tile kernels (VF_TMA=0 turns them off). On any failure
// the maps stay unused and the plain tile kernels run.
void make_tma_maps(vf_handle* h) {
  vf::TmaMaps& t = h->ad.tma;
  std::memset(&t, 0, sizeof(t));
  if (h->elem != 8) return;
  if (const char* e = std::getenv("VF_TMA"))
    if (std::strcmp(e, "0") == 0) return;
  const long long nxp = vf::XOFF + h->N1;  // columns 0..XOFF-1 are padding
  bool ok = true;
  for (int k = 0; k < 2; ++k) {
    ok = ok && encode_f64(&t.U[k], h->U[k], nxp, h->N2, h->P, h->PS, 3, vf::HX, vf::HY);
    // tile stores: extent ends at the last interior row and at or before the last interior column
    ok = ok && encode_f64(&t.Ust[k], h->U[k], vf::tma_store_cols(vf::XOFF + h->cfg.gc + h->cfg.nx),
                          h->cfg.gc + h->cfg.ny, h->P, h->PS, 3, vf::TX, vf::TY);
    t.Ub[k] = h->U[k];
  }
  ok = ok && encode_f64(&t.L, h->L, nxp, h->N2, h->P, h->PS, 3, vf::HX, vf::HY);
  t.Lb = h->L;
  if (h->S) ok = ok && encode_f64(&t.S, h->S, nxp, h->N2, h->P, h->PS, 1, vf::HX, vf::HY);
  t.Sb = h->S;
  if (h->B) ok = ok && encode_f64(&t.B, h->B, nxp + 1, h->N2 + 1, h->PB, 0, 1, vf::BHX, vf::BHY);
  t.Bb = h->B;
  t.ok = ok ? 1 : 0;
}

// Column marching covers wall BCs, linear reconstruction and constant sources;
// everything else runs on the tile kernels.
void select_variants(vf_handle* h) {
  const bool march_ok = h->cfg.bc == VF_BC_WALL && h->ad.p.rec_none == 0 && h->ad.p.any_dynamic == 0;
  h->ad.variant = 1;
  h->af.variant = march_ok ? 0 : 1;
  if (const char* kv = std::getenv("VF_KERNELS")) {
    if (std::strcmp(kv, "tile") == 0) h->ad.variant = h->af.variant = 1;
    if (std::strcmp(kv, "march") == 0 && march_ok) h->ad.variant = h->af.variant = 0;
  }
}

void refresh_params(vf_handle* h) {
  fill_phys(h, h->ad.p);
  fill_phys(h, h->af.p);
  select_variants(h);
  h->chunk_k = 0;  // a captured step chunk holds the old parameters
}

int validate(const vf_config* c) {
  if (!c) return fail(nullptr, VF_EINVAL, "config is NULL");
  if (c->abi_version != VF_ABI_VERSION) return fail(nullptr, VF_EINVAL, "abi_version mismatch");
  if (c->gc != 2)
    return fail(nullptr, VF_EINVAL, "gc must be 2 (LinearReconstruction needs gc > 1; the kernels stage a 2-cell halo)");
  if (c->nx < 2 || c->ny < 2) return fail(nullptr, VF_EINVAL, "nx and ny must be >= 2 for the wall mirror");
  if ((long long)c->nx * c->ny > (1ll << 31)) return fail(nullptr, VF_EINVAL, "grid too large");
  if (!(c->extent[1] > c->extent[0]) || !(c->extent[3] > c->extent[2]))
    return fail(nullptr, VF_EINVAL, "extent must be increasing");
  if (c->real_bytes != 8 && c->real_bytes != 4) return fail(nullptr, VF_EINVAL, "real_bytes must be 8 or 4");
  if (c->reconstruction != VF_REC_LINEAR && c->reconstruction != VF_REC_NONE)
    return fail(nullptr, VF_EINVAL, "reconstruction must be LinearReconstruction or NoReconstruction");
  if (c->stepper != VF_STEPPER_FE && c->stepper != VF_STEPPER_RK2)
    return fail(nullptr, VF_EINVAL, "stepper must be ForwardEuler or RungeKutta2");
  if (c->bc != VF_BC_WALL && c->bc != VF_BC_PERIODIC && c->bc != VF_BC_NEUMANN)
    return fail(nullptr, VF_EINVAL, "boundary must be WallBC, PeriodicBC or NeumannBC");
  if (!(c->desingularizing_kappa > 0) || !(c->depth_cutoff >= 0))
    return fail(nullptr, VF_EINVAL, "desingularizing_kappa must be positive and depth_cutoff non-negative");
  if (c->friction < VF_FRICTION_NONE || c->friction > VF_FRICTION_BH2021)
    return fail(nullptr, VF_EINVAL, "unknown friction law");
  if (c->n_sources < 0 || c->n_sources > VF_MAX_SOURCES) return fail(nullptr, VF_EINVAL, "too many source terms");
  bool has_bottom_source = false;
  for (int i = 0; i < c->n_sources; ++i) {
    const int k = c->source_kind[i];
    if (k < VF_SRC_BOTTOM || k > VF_SRC_RAIN_FIELD) return fail(nullptr, VF_EINVAL, "unknown source term");
    if (k == VF_SRC_BOTTOM) has_bottom_source = true;
  }
  // is_compatible, src/equations/equation.jl:74-84.
  if (c->bottom_is_constant && c->bottom_constant != 0.0 && !has_bottom_source)
    return fail(nullptr, VF_EINVAL,
                "Found non-zero bottom topography in equation, but no corresponding source term. Did you forget to add "
                "a source term to your system?");
  if (!(c->cfl > 0)) return fail(nullptr, VF_EINVAL, "cfl must be positive");
  return VF_OK;
}

void* plane(void* base, size_t elem, long long k, long long PS) {
  return static_cast<char*>(base) + (size_t)(k * PS) * elem;
}

// Copies between a dense host plane block (x fastest) and the padded device layout.
int copy_planes(vf_handle* h, void* dev, const void* host_src, void* host_dst, int x_first, int y_first, int w, int hgt,
                int planes, const void* const* host_planes_src, void* const* host_planes_dst) {
  const size_t e = h->elem;
  for (int k = 0; k < planes; ++k) {
    char* d = static_cast<char*>(plane(dev, e, k, h->PS)) + (size_t)((long long)y_first * h->P + x_first + vf::XOFF) * e;
    if (host_src || host_planes_src) {
      const char* s = host_planes_src ? static_cast<const char*>(host_planes_src[k])
                                      : static_cast<const char*>(host_src) + (size_t)k * w * hgt * e;
      if (!s) continue;
      VF_CK(h, cudaMemcpy2DAsync(d, (size_t)h->P * e, s, (size_t)w * e, (size_t)w * e, hgt, cudaMemcpyHostToDevice,
                                 h->stream));
    } else {
      char* o = host_planes_dst ? static_cast<char*>(host_planes_dst[k])
                                : static_cast<char*>(host_dst) + (size_t)k * w * hgt * e;
      if (!o) continue;
      VF_CK(h, cudaMemcpy2DAsync(o, (size_t)w * e, d, (size_t)h->P * e, (size_t)w * e, hgt, cudaMemcpyDeviceToHost,
                                 h->stream));
    }
  }
  return VF_OK;
}

int launch_one_step(vf_handle* h, int k) {
  const int parity = k & 1;
  cudaError_t e;
  if (h->elem == 8) {
    e = vf::launch_step(h->ad, static_cast<const double*>(h->U[parity]), static_cast<double*>(h->U[parity ^ 1]),
                        parity, h->stream);
  } else {
    e = vf::launch_step(h->af, static_cast<const float*>(h->U[parity]), static_cast<float*>(h->U[parity ^ 1]), parity,
                        h->stream);
  }
  h->launches += 2;
  if (e != cudaSuccess) return cuda_fail(h, e, "step launch");
  return VF_OK;
}

int push_record(vf_handle* h) {
  VF_CK(h, cudaMemcpyAsync(h->rec, h->rec_h, sizeof(vf::StepRecord), cudaMemcpyHostToDevice, h->stream));
  return VF_OK;
}

int pull_record(vf_handle* h) {
  VF_CK(h, cudaMemcpyAsync(h->rec_h, h->rec, sizeof(vf::StepRecord), cudaMemcpyDeviceToHost, h->stream));
  VF_CK(h, cudaStreamSynchronize(h->stream));
  if (h->rec_h->wait_fault)  // the block still loaded its tile the plain way, but the copy engine stalled for seconds
    return fail(h, VF_ECUDA, "a bounded wait for a TMA tile copy gave up (the tile was then loaded with plain loads)");
  return VF_OK;
}

void reset_record(vf_handle* h) {
  std::memset(h->rec_h, 0, sizeof(vf::StepRecord));
  h->rec_h->stop_time = std::numeric_limits<double>::infinity();
  h->rec_h->endtime = std::numeric_limits<double>::infinity();
}

int ensure_ready(vf_handle* h) {
  if (!h) return VF_EINVAL;
  if (!h->have_state) return fail(h, VF_ESTATE, "no state uploaded (call vf_set_interior_state first)");
  if (!h->cfg.bottom_is_constant && !h->have_bottom) return fail(h, VF_ESTATE, "bottom topography not uploaded");
  for (int i = 0; i < h->cfg.n_sources; ++i) {
    const int k = h->cfg.source_kind[i];
    if (k == VF_SRC_TIME_RAIN && !h->src_tab[i]) return fail(h, VF_ESTATE, "TimeDependentRain table not uploaded");
    if ((k == VF_SRC_HORTON || k == VF_SRC_RAIN_FIELD) && !h->src_field[i])
      return fail(h, VF_ESTATE, "source field not uploaded");
  }
  VF_CK(h, cudaSetDevice(h->device));
  return VF_OK;
}

void destroy(vf_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) {
    cudaStreamSynchronize(h->stream);
    dfree(h, h->U[0]);
    dfree(h, h->U[1]);
    dfree(h, h->L);
    dfree(h, h->S);
    dfree(h, h->B);
    dfree(h, h->rec);
    dfree(h, h->partial);
    dfree(h, h->vol_out);
    dfree(h, h->sample_ij);
    dfree(h, h->sample_out);
    for (int i = 0; i < VF_MAX_SOURCES; ++i) {
      dfree(h, h->src_field[i]);
      dfree(h, h->src_tab[i]);
    }
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
  }
  if (h->chunk_exec) cudaGraphExecDestroy(h->chunk_exec);
  delete h->rec_h;
  delete h;
}

}  // namespace

namespace vf {
int handle_ready(vf_handle* h) { return ensure_ready(h); }

int handle_begin_loop(vf_handle* h, double t0, double endtime, int match_endtime, double maximum_timestep) {
  reset_record(h);
  vf::StepRecord* r = h->rec_h;
  r->t[0] = t0;
  r->active[0] = t0 < endtime ? 1 : 0;
  r->match_endtime = match_endtime ? 1 : 0;
  r->has_max_ts = maximum_timestep >= 0 ? 1 : 0;
  r->max_ts = maximum_timestep;
  r->endtime = endtime;
  return push_record(h);
}

int handle_enqueue_steps(vf_handle* h, long long first, int n) {
  for (int i = 0; i < n; ++i)
    if (int rc = launch_one_step(h, (int)((first + i) & 1))) return rc;
  return VF_OK;
}

int handle_enqueue_chunk(vf_handle* h, int k) {
  if (!h->chunk_exec || h->chunk_k != k || h->chunk_u0 != h->U[0]) {
    if (h->chunk_exec) {
      cudaGraphExecDestroy(h->chunk_exec);
      h->chunk_exec = nullptr;
    }
    VF_CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = h->launches;
    int rc = handle_enqueue_steps(h, 0, k);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    h->launches = before;
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "step chunk capture");
    e = cudaGraphInstantiate(&h->chunk_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      h->chunk_exec = nullptr;
      return cuda_fail(h, e, "step chunk instantiation");
    }
    h->chunk_k = k;
    h->chunk_u0 = h->U[0];
  }
  VF_CK(h, cudaGraphLaunch(h->chunk_exec, h->stream));
  h->launches += 2LL * k;
  return VF_OK;
}

size_t handle_device_bytes(const vf_config* c) {
  const long long N1 = c->nx + 2LL * c->gc, N2 = c->ny + 2LL * c->gc;
  const long long P = round_up(vf::XOFF + N1, 32), PS = P * N2, PB = round_up(vf::XOFF + N1 + 1, 32);
  const size_t e = (size_t)c->real_bytes;
  size_t b = 3 * (size_t)(3 * PS) * e;                    // U[0], U[1], L
  if (c->friction != VF_FRICTION_NONE) b += (size_t)PS * e;
  if (!c->bottom_is_constant) b += (size_t)(PB * (N2 + 1)) * e;
  b += sizeof(vf::StepRecord) + sizeof(double) * 1025;    // record, volume partials and result
  return b;
}
}  // namespace vf

namespace {
// One warp waits on an mbarrier that thread 0 completes (arrive) or that
// nothing completes; *gave_up = 1 when any thread's bounded wait ran out.
__global__ void k_selftest_tile_wait(int arrive, int iterations, int* gave_up) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) vf::mbar_init(&bar, 1);
  __syncthreads();
  if (arrive && threadIdx.x == 0) vf::mbar_arrive(&bar);
  if (!vf::mbar_wait_bounded(&bar, 0, iterations)) atomicOr(gave_up, 1);
}
}  // namespace

extern "C" {

int vf_create(const vf_config* cfg, vf_handle** out) {
  if (!out) return fail(nullptr, VF_EINVAL, "out is NULL");
  *out = nullptr;
  int rc = validate(cfg);
  if (rc) return rc;
  vf_handle* h = new (std::nothrow) vf_handle();
  if (!h) return fail(nullptr, VF_ENOMEM, "host allocation failed");
  h->cfg = *cfg;
  h->device = cfg->device;
  h->elem = (size_t)cfg->real_bytes;
  h->N1 = cfg->nx + 2 * cfg->gc;
  h->N2 = cfg->ny + 2 * cfg->gc;
  // Rows padded to 32 elements with XOFF leading columns so interior rows start
  // 16-byte aligned; planes padded to whole rows of 32 elements.
  h->P = round_up(vf::XOFF + h->N1, 32);
  h->PS = h->P * h->N2;
  h->PB = round_up(vf::XOFF + h->N1 + 1, 32);
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(nullptr, e, "cudaSetDevice");
  }
  e = h->elem == 8 ? vf::configure_kernels_f64() : vf::configure_kernels_f32();
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(nullptr, e, "kernel configuration");
  }
  const size_t state_bytes = (size_t)(3 * h->PS) * h->elem;
  bool ok = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && dalloc(h, &h->U[0], state_bytes);
  ok = ok && dalloc(h, &h->U[1], state_bytes);
  ok = ok && dalloc(h, &h->L, state_bytes);
  if (cfg->friction != VF_FRICTION_NONE) ok = ok && dalloc(h, &h->S, (size_t)h->PS * h->elem);
  if (!cfg->bottom_is_constant) ok = ok && dalloc(h, &h->B, (size_t)(h->PB * (h->N2 + 1)) * h->elem);
  ok = ok && dalloc(h, reinterpret_cast<void**>(&h->rec), sizeof(vf::StepRecord));
  h->rec_h = new (std::nothrow) vf::StepRecord();
  ok = ok && h->rec_h != nullptr;
  h->vol_blocks = 1024;
  ok = ok && dalloc(h, reinterpret_cast<void**>(&h->partial), sizeof(double) * h->vol_blocks);
  ok = ok && dalloc(h, reinterpret_cast<void**>(&h->vol_out), sizeof(double));
  if (!ok) {
    cudaGetLastError();
    destroy(h);
    return fail(nullptr, VF_ENOMEM, "device allocation failed");
  }
  ok = cudaMemsetAsync(h->U[0], 0, state_bytes, h->stream) == cudaSuccess;
  ok = ok && cudaMemsetAsync(h->U[1], 0, state_bytes, h->stream) == cudaSuccess;
  ok = ok && cudaMemsetAsync(h->L, 0, state_bytes, h->stream) == cudaSuccess;
  if (h->S) ok = ok && cudaMemsetAsync(h->S, 0, (size_t)h->PS * h->elem, h->stream) == cudaSuccess;
  if (h->B) ok = ok && cudaMemsetAsync(h->B, 0, (size_t)(h->PB * (h->N2 + 1)) * h->elem, h->stream) == cudaSuccess;
  ok = ok && cudaMemsetAsync(h->rec, 0, sizeof(vf::StepRecord), h->stream) == cudaSuccess;
  ok = ok && cudaStreamSynchronize(h->stream) == cudaSuccess;
  if (!ok) {
    cudaError_t le = cudaGetLastError();
    destroy(h);
    return cuda_fail(nullptr, le, "device initialisation");
  }
  fill_geom(h, h->ad.g);
  fill_geom(h, h->af.g);
  refresh_params(h);
  h->ad.rk2 = h->af.rk2 = cfg->stepper == VF_STEPPER_RK2;
  // Default kernels per precision: shared-memory tiles for Float64 (full warps on the
  // 1/64-rate FP64 pipe), column marching for Float32 (fewest instructions per cell)
  // where it applies; VF_KERNELS=tile|march overrides (select_variants).
  h->ad.B = static_cast<const double*>(h->B);
  h->ad.L = static_cast<double*>(h->L);
  h->ad.S = static_cast<double*>(h->S);
  h->ad.rec = h->rec;
  h->af.B = static_cast<const float*>(h->B);
  h->af.L = static_cast<float*>(h->L);
  h->af.S = static_cast<float*>(h->S);
  h->af.rec = h->rec;
  h->ad.arith = h->af.arith = VF_ARITH_REFERENCE;
  make_tma_maps(h);
  *out = h;
  return VF_OK;
}

int vf_set_arithmetic(vf_handle* h, int32_t mode) {
  if (!h) return fail(nullptr, VF_EINVAL, "handle is NULL");
  if (mode != VF_ARITH_REFERENCE && mode != VF_ARITH_FAITHFUL)
    return fail(h, VF_EINVAL, "arithmetic mode must be VF_ARITH_REFERENCE or VF_ARITH_FAITHFUL");
  if (h->elem != 8 && mode != VF_ARITH_REFERENCE)
    return fail(h, VF_EINVAL, "faithful arithmetic is a Float64 mode");
  h->ad.arith = mode;
  h->chunk_k = 0;  // a captured step chunk holds the old kernels
  return VF_OK;
}

void vf_destroy(vf_handle* h) { destroy(h); }

int vf_upload_bottom(vf_handle* h, const void* B_corners) {
  if (!h || !B_corners) return fail(h, VF_EINVAL, "NULL argument");
  if (h->cfg.bottom_is_constant) return fail(h, VF_EINVAL, "handle uses a ConstantBottomTopography");
  const long long W = h->N1 + 1, H = h->N2 + 1;
  // is_compatible, src/equations/equation.jl:74-84: non-zero B needs SourceTermBottom.
  bool has_bottom_source = false;
  for (int i = 0; i < h->cfg.n_sources; ++i) has_bottom_source |= h->cfg.source_kind[i] == VF_SRC_BOTTOM;
  if (!has_bottom_source) {
    for (long long n = 0; n < W * H; ++n) {
      const double v = h->elem == 8 ? static_cast<const double*>(B_corners)[n] : static_cast<const float*>(B_corners)[n];
      if (v != 0.0)
        return fail(h, VF_EINVAL,
                    "Found non-zero bottom topography in equation, but no corresponding source term. Did you forget to "
                    "add a source term to your system?");
    }
  }
  VF_CK(h, cudaSetDevice(h->device));
  char* d = static_cast<char*>(h->B) + (size_t)vf::XOFF * h->elem;
  VF_CK(h, cudaMemcpy2DAsync(d, (size_t)h->PB * h->elem, B_corners, (size_t)W * h->elem, (size_t)W * h->elem, H,
                             cudaMemcpyHostToDevice, h->stream));
  VF_CK(h, cudaStreamSynchronize(h->stream));
  h->have_bottom = true;
  return VF_OK;
}

int vf_set_source_table(vf_handle* h, int32_t index, const double* times, const double* rates, int32_t n) {
  if (!h || !times || !rates || n < 1) return fail(h, VF_EINVAL, "invalid table");
  if (index < 0 || index >= h->cfg.n_sources || h->cfg.source_kind[index] != VF_SRC_TIME_RAIN)
    return fail(h, VF_EINVAL, "source index is not a TimeDependentRain");
  VF_CK(h, cudaSetDevice(h->device));
  double* host = new (std::nothrow) double[2 * n];
  if (!host) return fail(h, VF_ENOMEM, "host allocation failed");
  for (int i = 0; i < n; ++i) {
    host[i] = times[i];
    host[n + i] = rates[i] / 3600;  // compute_rain, src/sourceterms/source_term_rain.jl:53
  }
  if (h->src_tab[index] && h->src_tab_n[index] != n) {
    dfree(h, h->src_tab[index]);
    h->src_tab[index] = nullptr;
  }
  cudaError_t e = cudaSuccess;
  if (!h->src_tab[index] && !dalloc(h, reinterpret_cast<void**>(&h->src_tab[index]), sizeof(double) * 2 * n))
    e = cudaErrorMemoryAllocation;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->src_tab[index], host, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  delete[] host;
  if (e != cudaSuccess) return cuda_fail(h, e, "source table upload");
  h->src_tab_n[index] = n;
  refresh_params(h);
  return VF_OK;
}

int vf_set_source_field(vf_handle* h, int32_t index, const void* field) {
  if (!h || !field) return fail(h, VF_EINVAL, "NULL argument");
  if (index < 0 || index >= h->cfg.n_sources ||
      (h->cfg.source_kind[index] != VF_SRC_HORTON && h->cfg.source_kind[index] != VF_SRC_RAIN_FIELD))
    return fail(h, VF_EINVAL, "source index is not a HortonInfiltration or rain field");
  VF_CK(h, cudaSetDevice(h->device));
  if (!h->src_field[index]) {
    if (!dalloc(h, &h->src_field[index], (size_t)h->PS * h->elem)) return fail(h, VF_ENOMEM, "device allocation failed");
    VF_CK(h, cudaMemsetAsync(h->src_field[index], 0, (size_t)h->PS * h->elem, h->stream));
  }
  int rc = copy_planes(h, h->src_field[index], field, nullptr, 0, 0, h->N1, h->N2, 1, nullptr, nullptr);
  if (rc) return rc;
  VF_CK(h, cudaStreamSynchronize(h->stream));
  refresh_params(h);
  return VF_OK;
}

int vf_set_interior_state(vf_handle* h, const void* w, const void* hu, const void* hv) {
  if (!h || !w || !hu || !hv) return fail(h, VF_EINVAL, "NULL argument");
  VF_CK(h, cudaSetDevice(h->device));
  const void* planes[3] = {w, hu, hv};
  int rc = copy_planes(h, h->U[0], nullptr, nullptr, h->cfg.gc, h->cfg.gc, h->cfg.nx, h->cfg.ny, 3, planes, nullptr);
  if (rc) return rc;
  cudaError_t e = h->elem == 8 ? vf::launch_bc(h->ad.g, static_cast<double*>(h->U[0]), h->stream)
                               : vf::launch_bc(h->af.g, static_cast<float*>(h->U[0]), h->stream);
  h->launches += 1;
  if (e != cudaSuccess) return cuda_fail(h, e, "boundary update");
  VF_CK(h, cudaStreamSynchronize(h->stream));
  h->have_state = true;
  return VF_OK;
}

int vf_upload_state(vf_handle* h, const void* state) {
  if (!h || !state) return fail(h, VF_EINVAL, "NULL argument");
  VF_CK(h, cudaSetDevice(h->device));
  int rc = copy_planes(h, h->U[0], state, nullptr, 0, 0, h->N1, h->N2, 3, nullptr, nullptr);
  if (rc) return rc;
  VF_CK(h, cudaStreamSynchronize(h->stream));
  h->have_state = true;
  return VF_OK;
}

int vf_download_state(vf_handle* h, void* state) {
  if (!h || !state) return fail(h, VF_EINVAL, "NULL argument");
  VF_CK(h, cudaSetDevice(h->device));
  int rc = copy_planes(h, h->U[0], nullptr, state, 0, 0, h->N1, h->N2, 3, nullptr, nullptr);
  if (rc) return rc;
  VF_CK(h, cudaStreamSynchronize(h->stream));
  return VF_OK;
}

int vf_get_interior_state(vf_handle* h, void* w, void* hu, void* hv) {
  if (!h) return VF_EINVAL;
  VF_CK(h, cudaSetDevice(h->device));
  void* planes[3] = {w, hu, hv};
  int rc = copy_planes(h, h->U[0], nullptr, nullptr, h->cfg.gc, h->cfg.gc, h->cfg.nx, h->cfg.ny, 3, nullptr, planes);
  if (rc) return rc;
  VF_CK(h, cudaStreamSynchronize(h->stream));
  return VF_OK;
}

int vf_step(vf_handle* h, double max_dt, double t, double* dt_out) {
  int rc = ensure_ready(h);
  if (rc) return rc;
  reset_record(h);
  h->rec_h->active[0] = 1;
  h->rec_h->t[0] = t;
  h->rec_h->explicit_mode = 1;
  h->rec_h->explicit_max_dt = max_dt;
  if ((rc = push_record(h))) return rc;
  if ((rc = launch_one_step(h, 0))) return rc;
  if ((rc = pull_record(h))) return rc;
  std::swap(h->U[0], h->U[1]);
  if (dt_out) *dt_out = h->rec_h->last_dt;
  return VF_OK;
}

int vf_step_fixed(vf_handle* h, double dt, double t) {
  int rc = ensure_ready(h);
  if (rc) return rc;
  if (!(dt >= 0)) return fail(h, VF_EINVAL, "dt must be >= 0");
  reset_record(h);
  h->rec_h->active[0] = 1;
  h->rec_h->t[0] = t;
  h->rec_h->explicit_mode = 1;
  h->rec_h->force_dt = 1;
  h->rec_h->forced_dt = dt;
  if ((rc = push_record(h))) return rc;
  if ((rc = launch_one_step(h, 0))) return rc;
  if ((rc = pull_record(h))) return rc;
  std::swap(h->U[0], h->U[1]);
  return VF_OK;
}

int vf_simulate(vf_handle* h, double t0, double endtime, int32_t match_endtime, double maximum_timestep,
                double stop_time, int64_t max_steps, double* t_out, int64_t* steps_out, double* last_dt_out) {
  int rc = ensure_ready(h);
  if (rc) return rc;
  reset_record(h);
  vf::StepRecord* r = h->rec_h;
  r->t[0] = t0;
  r->active[0] = t0 < endtime ? 1 : 0;
  r->match_endtime = match_endtime ? 1 : 0;
  r->has_max_ts = maximum_timestep >= 0 ? 1 : 0;
  r->max_ts = maximum_timestep;
  r->endtime = endtime;
  r->stop_time = stop_time;
  const bool limited = max_steps > 0;
  if ((rc = push_record(h))) return rc;
  long long k = 0;
  long long chunk = 8;
  if (r->active[0]) {
    for (;;) {
      long long n = chunk;
      if (limited && k + n > max_steps) n = max_steps - k;
      for (long long i = 0; i < n; ++i)
        if ((rc = launch_one_step(h, (int)((k + i) & 1)))) return rc;
      k += n;
      if ((rc = pull_record(h))) return rc;
      if (!h->rec_h->active[k & 1]) break;
      if (limited && k >= max_steps) break;
      if (chunk < 256) chunk *= 2;
    }
  }
  if (k == 0 && (rc = pull_record(h))) return rc;
  const long long done = h->rec_h->n_done;
  if (done & 1) std::swap(h->U[0], h->U[1]);
  if (t_out) *t_out = h->rec_h->t[k & 1];
  if (steps_out) *steps_out = done;
  if (last_dt_out) *last_dt_out = h->rec_h->last_dt;
  return VF_OK;
}

int vf_selftest_tile_wait(int32_t device, int32_t arrive, int32_t iterations, int32_t* gave_up) {
  if (!gave_up || iterations < 1 || iterations > (1 << 22))
    return fail(nullptr, VF_EINVAL, "gave_up must be non-NULL and iterations in [1, 2^22]");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  int* d = nullptr;
  if ((e = cudaMalloc(&d, sizeof(int))) != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  e = cudaMemset(d, 0, sizeof(int));
  if (e == cudaSuccess) {
    k_selftest_tile_wait<<<1, 32>>>(arrive ? 1 : 0, iterations, d);
    e = cudaGetLastError();
  }
  int v = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&v, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "tile-wait self-test");
  *gave_up = v;
  return VF_OK;
}

int vf_selftest_quotients(int32_t device, const double* a, const double* b, int32_t n, double* q) {
  if (!a || !b || !q || n < 1) return fail(nullptr, VF_EINVAL, "a, b, q must be non-NULL and n >= 1");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  double* d = nullptr;
  const size_t bytes = sizeof(double) * (size_t)n;
  if ((e = cudaMalloc(&d, 3 * bytes)) != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  e = cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = vf::launch_selftest_quotients(d, d + n, n, d + 2 * (size_t)n, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(q, d + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "quotient self-test");
  return VF_OK;
}

int vf_selftest_near_dry_quotients(int32_t device, const float* a, const float* b, int32_t n, float* q,
                                   float* q64) {
  if (!a || !b || !q || !q64 || n < 1) return fail(nullptr, VF_EINVAL, "a, b, q, q64 must be non-NULL and n >= 1");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  float* d = nullptr;
  const size_t bytes = sizeof(float) * (size_t)n;
  if ((e = cudaMalloc(&d, 4 * bytes)) != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  e = cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = vf::launch_selftest_near_dry(d, d + n, n, d + 2 * (size_t)n, d + 3 * (size_t)n, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(q, d + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(q64, d + 3 * (size_t)n, bytes, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "near-dry quotient self-test");
  return VF_OK;
}

int vf_time_steps(vf_handle* h, int64_t n_steps, float* ms_out) {
  int rc = ensure_ready(h);
  if (rc) return rc;
  if (n_steps < 1) return fail(h, VF_EINVAL, "n_steps must be >= 1");
  reset_record(h);
  h->rec_h->active[0] = 1;
  h->rec_h->t[0] = 0.0;
  if ((rc = push_record(h))) return rc;
  cudaEvent_t e0, e1;
  VF_CK(h, cudaEventCreate(&e0));
  VF_CK(h, cudaEventCreate(&e1));
  VF_CK(h, cudaEventRecord(e0, h->stream));
  for (long long k = 0; k < n_steps; ++k)
    if ((rc = launch_one_step(h, (int)(k & 1)))) return rc;
  VF_CK(h, cudaEventRecord(e1, h->stream));
  VF_CK(h, cudaEventSynchronize(e1));
  float ms = 0.f;
  VF_CK(h, cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if ((rc = pull_record(h))) return rc;
  if (h->rec_h->n_done & 1) std::swap(h->U[0], h->U[1]);
  if (ms_out) *ms_out = ms;
  return VF_OK;
}

int vf_time_kernels(vf_handle* h, int64_t n_steps, float* ms_flux, float* ms_stage) {
  int rc = ensure_ready(h);
  if (rc) return rc;
  if (n_steps < 1) return fail(h, VF_EINVAL, "n_steps must be >= 1");
  reset_record(h);
  h->rec_h->active[0] = 1;
  if ((rc = push_record(h))) return rc;
  const long long ne = 2 * n_steps + 1;
  cudaEvent_t* ev = new (std::nothrow) cudaEvent_t[ne];
  if (!ev) return fail(h, VF_ENOMEM, "host allocation failed");
  for (long long i = 0; i < ne; ++i) VF_CK(h, cudaEventCreate(&ev[i]));
  VF_CK(h, cudaEventRecord(ev[0], h->stream));
  for (long long k = 0; k < n_steps; ++k) {
    const int parity = (int)(k & 1);
    cudaError_t e;
    if (h->elem == 8) {
      e = vf::launch_flux(h->ad, static_cast<const double*>(h->U[parity]), parity, h->stream);
      if (e == cudaSuccess) e = cudaEventRecord(ev[2 * k + 1], h->stream);
      if (e == cudaSuccess)
        e = vf::launch_stage(h->ad, static_cast<const double*>(h->U[parity]), static_cast<double*>(h->U[parity ^ 1]),
                             parity, h->stream);
    } else {
      e = vf::launch_flux(h->af, static_cast<const float*>(h->U[parity]), parity, h->stream);
      if (e == cudaSuccess) e = cudaEventRecord(ev[2 * k + 1], h->stream);
      if (e == cudaSuccess)
        e = vf::launch_stage(h->af, static_cast<const float*>(h->U[parity]), static_cast<float*>(h->U[parity ^ 1]),
                             parity, h->stream);
    }
    h->launches += 2;
    if (e == cudaSuccess) e = cudaEventRecord(ev[2 * k + 2], h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "timed step");
  }
  VF_CK(h, cudaEventSynchronize(ev[ne - 1]));
  float f = 0.f, s = 0.f;
  for (long long k = 0; k < n_steps; ++k) {
    float a = 0.f, b = 0.f;
    VF_CK(h, cudaEventElapsedTime(&a, ev[2 * k], ev[2 * k + 1]));
    VF_CK(h, cudaEventElapsedTime(&b, ev[2 * k + 1], ev[2 * k + 2]));
    f += a;
    s += b;
  }
  for (long long i = 0; i < ne; ++i) cudaEventDestroy(ev[i]);
  delete[] ev;
  if ((rc = pull_record(h))) return rc;
  if (h->rec_h->n_done & 1) std::swap(h->U[0], h->U[1]);
  if (ms_flux) *ms_flux = f;
  if (ms_stage) *ms_stage = s;
  return VF_OK;
}

int vf_water_volume(vf_handle* h, double* out) {
  int rc = ensure_ready(h);
  if (rc) return rc;
  if (!out) return fail(h, VF_EINVAL, "NULL argument");
  cudaError_t e = h->elem == 8
                      ? vf::launch_volume(h->ad.g, static_cast<const double*>(h->U[0]),
                                          static_cast<const double*>(h->B), h->partial, h->vol_blocks, h->vol_out,
                                          h->stream)
                      : vf::launch_volume(h->af.g, static_cast<const float*>(h->U[0]), static_cast<const float*>(h->B),
                                          h->partial, h->vol_blocks, h->vol_out, h->stream);
  h->launches += 2;
  if (e != cudaSuccess) return cuda_fail(h, e, "volume launch");
  VF_CK(h, cudaMemcpyAsync(out, h->vol_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  VF_CK(h, cudaStreamSynchronize(h->stream));
  return VF_OK;
}

int vf_sample_cells(vf_handle* h, const int32_t* i, const int32_t* j, int32_t n, void* w_out, void* hu_out,
                    void* hv_out) {
  int rc = ensure_ready(h);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!i || !j))) return fail(h, VF_EINVAL, "bad gauge list");
  if (n == 0) return VF_OK;
  for (int k = 0; k < n; ++k)
    if (i[k] < 0 || j[k] < 0 || i[k] >= h->cfg.nx || j[k] >= h->cfg.ny) return fail(h, VF_EINVAL, "gauge outside the grid");
  if (n > h->sample_cap) {
    dfree(h, h->sample_ij);
    dfree(h, h->sample_out);
    h->sample_ij = nullptr;
    h->sample_out = nullptr;
    h->sample_cap = 0;
    if (!dalloc(h, reinterpret_cast<void**>(&h->sample_ij), sizeof(int) * 2 * (size_t)n) ||
        !dalloc(h, &h->sample_out, h->elem * 3 * (size_t)n))
      return fail(h, VF_ENOMEM, "device allocation failed");
    h->sample_cap = n;
  }
  VF_CK(h, cudaMemcpyAsync(h->sample_ij, i, sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
  VF_CK(h, cudaMemcpyAsync(h->sample_ij + n, j, sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
  cudaError_t e = h->elem == 8 ? vf::launch_sample(h->ad.g, static_cast<const double*>(h->U[0]), h->sample_ij, n,
                                                   static_cast<double*>(h->sample_out), h->stream)
                               : vf::launch_sample(h->af.g, static_cast<const float*>(h->U[0]), h->sample_ij, n,
                                                   static_cast<float*>(h->sample_out), h->stream);
  h->launches += 1;
  if (e != cudaSuccess) return cuda_fail(h, e, "sample launch");
  void* outs[3] = {w_out, hu_out, hv_out};
  for (int k = 0; k < 3; ++k)
    if (outs[k])
      VF_CK(h, cudaMemcpyAsync(outs[k], static_cast<char*>(h->sample_out) + (size_t)k * n * h->elem, h->elem * n,
                               cudaMemcpyDeviceToHost, h->stream));
  VF_CK(h, cudaStreamSynchronize(h->stream));
  return VF_OK;
}

int vf_device_state(vf_handle* h, void** base, int64_t* pitch, int64_t* plane_stride, int64_t* offset00) {
  if (!h) return VF_EINVAL;
  if (base) *base = h->U[0];
  if (pitch) *pitch = h->P;
  if (plane_stride) *plane_stride = h->PS;
  if (offset00) *offset00 = vf::XOFF;
  return VF_OK;
}

int vf_stream(vf_handle* h, void** stream) {
  if (!h || !stream) return VF_EINVAL;
  *stream = h->stream;
  return VF_OK;
}

const char* vf_last_error(vf_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int64_t vf_launch_count(vf_handle* h) { return h ? h->launches : 0; }

}  // extern "C"
