// vf_batch.cu -- the batched-ensemble entry points (vf_batch_*) of
// include/volumefluxes_sm103.h.
//
// A batch takes handles that are ready to step and runs the time loop of each
// on the device in k_ensemble (vf_ensemble.cuh): one thread-block cluster per
// simulation, clusters sized from the simulation's tile count, one launch per
// (precision, cluster size) group on its own stream so the groups overlap.
// Simulations are ordered largest estimated work first inside a launch, which
// the block scheduler then starts in that order (longest-processing-time
// first). Each cluster writes its result and a done flag into pinned, mapped
// host memory, so the host sees every simulation finish without synchronising
// the launch it belongs to.
//
// Simulations of at least wide_cells interior cells (default 512^2) are
// "wide": a 16-CTA cluster would leave most of the GPU to them alone and make
// them the batch's tail, so they run the plain
// whole-grid step kernels on their handle's stream instead, as the device loop
// of vf_simulate, in chunks of kChunk steps captured once as a CUDA graph.
// kInFlight chunks are kept queued; after each, the step record is copied to pinned
// memory behind an event, and the host retires chunks and enqueues new ones
// whenever the batch is polled. Their kernels share the SMs with the cluster
// launches, and their results are those of vf_simulate.
//
// Nothing here allocates with cudaMalloc, cudaFree or cudaFreeHost, which may
// synchronise the whole device: launch descriptors come from the library's
// stream-ordered pool and result slots from a pinned slab kept for the life of
// the process.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "vf_handle.h"

namespace {
// A wide member: the plain device loop on its handle's stream, fed in chunks.
struct Wide {
  int member = 0;
  long long enqueued = 0;      // steps enqueued so far
  long long max_steps = 0;
  int head = 0, inflight = 0;  // chunks head .. head+inflight-1 are in flight; chunk c uses ev/rec slot c % 3
  long long chunk_end[3] = {0, 0, 0};
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  double last_t = 0;
  bool done = false;
};
}  // namespace

struct vf_batch {
  int device = 0;
  int n = 0;
  std::vector<Wide> wide;
  std::chrono::steady_clock::time_point start;
  double time_limit_s = 0;
  std::vector<vf_handle*> hs;
  std::vector<cudaStream_t> streams;
  std::vector<int> slots;          // result slot of simulation i
  std::vector<char> collected;
  void* items_d[2] = {nullptr, nullptr};  // EnsItem<double>[], EnsItem<float>[]
  int* order_d = nullptr;
  unsigned long long* epoch_d = nullptr;  // watchdog start of the batch
  cudaStream_t setup = nullptr;    // stream of the descriptor copies (streams[0])
  std::string err;
};

namespace {

thread_local std::string g_batch_error;

int bfail(vf_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  else g_batch_error = msg;
  return code;
}

// ---- result slots: pinned, device-mapped, never freed ---------------------
// A slot holds the result a cluster writes (res) and, for wide members, the
// two step-record copies of the chunks in flight.
struct Slot {
  vf::EnsResult res;
  vf::StepRecord rec[3];
};

constexpr int kSlab = 4096;
std::mutex g_slot_mu;
std::vector<Slot*> g_slabs;  // host pointers
std::vector<Slot*> g_slabs_d;
std::vector<int> g_free_slots;

int acquire_slots(int n, std::vector<int>& out, std::string& err) {
  std::lock_guard<std::mutex> lk(g_slot_mu);
  while ((int)g_free_slots.size() < n) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, sizeof(Slot) * kSlab, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
      cudaGetLastError();
      err = "pinned result slab allocation failed";
      return VF_ENOMEM;
    }
    void* d = nullptr;
    if (cudaHostGetDevicePointer(&d, p, 0) != cudaSuccess) {
      cudaGetLastError();
      err = "mapped result slab has no device address";
      return VF_ECUDA;
    }
    const int base = (int)g_slabs.size() * kSlab;
    g_slabs.push_back(static_cast<Slot*>(p));
    g_slabs_d.push_back(static_cast<Slot*>(d));
    for (int i = kSlab - 1; i >= 0; --i) g_free_slots.push_back(base + i);
  }
  out.resize(n);
  for (int i = 0; i < n; ++i) {
    out[i] = g_free_slots.back();
    g_free_slots.pop_back();
  }
  return VF_OK;
}

void release_slots(const std::vector<int>& s) {
  std::lock_guard<std::mutex> lk(g_slot_mu);
  for (int v : s) g_free_slots.push_back(v);
}

vf::EnsResult* slot_host(int s) { return &(g_slabs[s / kSlab] + s % kSlab)->res; }
vf::EnsResult* slot_dev(int s) { return &(g_slabs_d[s / kSlab] + s % kSlab)->res; }
vf::StepRecord* slot_rec(int s, int k) { return &(g_slabs[s / kSlab] + s % kSlab)->rec[k]; }

int slot_done(int s) { return __atomic_load_n(&slot_host(s)->done, __ATOMIC_ACQUIRE); }

// ---- cluster sizing ---------------------------------------------------------
struct Opts {
  int tiles_per_cta;
  int max_cluster;
  double time_limit_s;
  int seg_rows;  // 0: heuristic
  long long wide_cells;
};

Opts resolve(const vf_batch_options* o) {
  Opts r{16, 16, 600.0, 0, 1LL << 18};
  if (o) {
    if (o->wide_cells > 0) r.wide_cells = o->wide_cells;
    if (o->wide_cells < 0) r.wide_cells = LLONG_MAX;
    if (o->tiles_per_cta > 0) r.tiles_per_cta = o->tiles_per_cta;
    if (o->max_cluster > 0) r.max_cluster = std::min(16, o->max_cluster);
    if (o->time_limit_s > 0) r.time_limit_s = o->time_limit_s;
    if (o->seg_rows > 0) r.seg_rows = std::min(256, std::max(8, o->seg_rows));
  }
  return r;
}

// Kernel design of a member, as the plain path chooses it (vf_abi.cu
// select_variants): column marching for Float32 members with wall BCs, linear
// reconstruction and constant sources (0 with RK2, 2 with forward Euler);
// tiles (1) for everything else.
int variant_of(const vf_handle* h) {
  if (h->elem == 4 && h->af.variant == 0) return h->af.rk2 ? 0 : 2;
  return 1;
}

// Largest launchable cluster size <= c on the current device.
std::mutex g_fit_mu;
int g_fit[64][2][3][17];  // [device][precision][variant][c]: 0 unknown, else 1 + launchable

int fit_cluster(int device, int real_bytes, int variant, int c) {
  const int pi = real_bytes == 8 ? 0 : 1;
  for (; c > 1; c /= 2) {
    int ok;
    {
      std::lock_guard<std::mutex> lk(g_fit_mu);
      ok = device < 64 ? g_fit[device][pi][variant][c] : 0;
    }
    if (!ok) {
      int nclusters = 0;
      cudaError_t e = real_bytes == 8 ? vf::ensemble_max_clusters_f64(c, variant, &nclusters)
                                      : vf::ensemble_max_clusters_f32(c, variant, &nclusters);
      if (e != cudaSuccess) cudaGetLastError();
      ok = (e == cudaSuccess && nclusters > 0) ? 2 : 1;
      std::lock_guard<std::mutex> lk(g_fit_mu);
      if (device < 64) g_fit[device][pi][variant][c] = ok;
    }
    if (ok == 2) return c;
  }
  return 1;
}

// Rows per strip segment of a marching member: 64, halved (down to 8) until
// the cluster's warps have at least two segments each.
int seg_rows_for(const vf_handle* h, int csize, int fixed) {
  if (fixed > 0) return fixed;
  const int nstrips = (h->cfg.nx + vf::MOUT - 1) / vf::MOUT;
  int seg = 64;
  while (seg > 8 && (long long)nstrips * ((h->cfg.ny + seg - 1) / seg) < 2LL * csize * (vf::NT / 32)) seg /= 2;
  return seg;
}

int cluster_for(const vf_handle* h, const Opts& o) {
  const long long tiles =
      (long long)((h->cfg.nx + vf::TX - 1) / vf::TX) * ((h->cfg.ny + vf::TY - 1) / vf::TY);
  int c = 1;
  while (c < o.max_cluster && (long long)c * o.tiles_per_cta < tiles) c *= 2;
  return std::min(c, o.max_cluster);
}

template <typename T>
vf::EnsItem<T> make_item(vf_handle* h, const vf::StepArgs<T>& a, double t0, double endtime, int match,
                         double max_ts, long long max_steps, vf::EnsResult* res, unsigned long long* epoch) {
  vf::EnsItem<T> it;
  std::memset(&it, 0, sizeof(it));
  it.g = a.g;
  it.p = a.p;
  it.B = a.B;
  it.U[0] = static_cast<T*>(h->U[0]);
  it.U[1] = static_cast<T*>(h->U[1]);
  it.L = a.L;
  it.S = a.S;
  it.t0 = t0;
  it.endtime = endtime;
  it.max_ts = max_ts;
  it.match_endtime = match ? 1 : 0;
  it.has_max_ts = max_ts >= 0 ? 1 : 0;
  it.rk2 = a.rk2;
  it.max_steps = max_steps > 0 ? max_steps : LLONG_MAX;
  it.res = res;
  it.epoch = epoch;
  return it;
}

void destroy_batch(vf_batch* b) {
  if (!b) return;
  if (b->setup) {
    cudaFreeAsync(b->items_d[0], b->setup);
    cudaFreeAsync(b->items_d[1], b->setup);
    cudaFreeAsync(b->order_d, b->setup);
    cudaFreeAsync(b->epoch_d, b->setup);
  }
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  for (Wide& w : b->wide)
    for (cudaEvent_t e : w.ev)
      if (e) cudaEventDestroy(e);
  release_slots(b->slots);
  delete b;
}

constexpr int kChunk = 16;    // steps per graph launch of a wide member
constexpr int kInFlight = 3;  // chunks kept queued per wide member (rides out host stalls)

// Final result of a wide member from the record copy of its last retired chunk.
void wide_finish(vf_batch* b, Wide& w, const vf::StepRecord& r, long long k, int status) {
  vf_handle* h = b->hs[w.member];
  cudaStreamSynchronize(h->stream);  // no-op steps of a chunk still in flight
  vf::EnsResult* res = slot_host(b->slots[w.member]);
  res->t = r.t[k & 1];
  res->last_dt = r.last_dt;
  res->steps = r.n_done;
  res->status = status;
  w.done = true;
  __atomic_store_n(&res->done, 1, __ATOMIC_RELEASE);
}

int wide_enqueue(vf_batch* b, Wide& w) {
  vf_handle* h = b->hs[w.member];
  const long long left = w.max_steps - w.enqueued;
  const int n = (int)std::min<long long>(kChunk, left);
  int rc = (n == kChunk && (w.enqueued & 1) == 0) ? vf::handle_enqueue_chunk(h, kChunk)
                                                  : vf::handle_enqueue_steps(h, w.enqueued, n);
  if (rc) return rc;
  w.enqueued += n;
  const int slot = (w.head + w.inflight) % kInFlight;
  cudaError_t e = cudaMemcpyAsync(slot_rec(b->slots[w.member], slot), h->rec, sizeof(vf::StepRecord),
                                  cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaEventRecord(w.ev[slot], h->stream);
  if (e != cudaSuccess) return VF_ECUDA;
  w.chunk_end[slot] = w.enqueued;
  w.inflight += 1;
  return VF_OK;
}

// Retire finished chunks of every wide member and keep two in flight.
int pump(vf_batch* b) {
  if (b->wide.empty()) return VF_OK;
  const double elapsed =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - b->start).count();
  const bool late = elapsed > b->time_limit_s;
  for (Wide& w : b->wide) {
    if (w.done) continue;
    while (w.inflight > 0) {
      const int slot = w.head % kInFlight;
      const cudaError_t q = cudaEventQuery(w.ev[slot]);
      if (q == cudaErrorNotReady) break;
      if (q != cudaSuccess) return bfail(b, VF_ECUDA, std::string("wide member: ") + cudaGetErrorString(q));
      const vf::StepRecord& r = *slot_rec(b->slots[w.member], slot);
      const long long k = w.chunk_end[slot];
      w.head += 1;
      w.inflight -= 1;
      if (r.wait_fault)
        return bfail(b, VF_ECUDA, "wide member: a bounded wait for a TMA tile copy gave up");
      if (!r.active[k & 1]) {
        wide_finish(b, w, r, k, vf::kEnsOk);
        break;
      }
      if (k >= w.max_steps) {
        wide_finish(b, w, r, k, vf::kEnsMaxSteps);
        break;
      }
      if (r.t[k & 1] == w.last_t && k > 0) {  // a whole chunk without progress
        wide_finish(b, w, r, k, vf::kEnsStalled);
        break;
      }
      w.last_t = r.t[k & 1];
      if (late && w.inflight == 0) {
        wide_finish(b, w, r, k, vf::kEnsTimeout);
        break;
      }
    }
    if (!w.done && late && w.inflight == 0) {
      const int last = (w.head + kInFlight - 1) % kInFlight;
      wide_finish(b, w, *slot_rec(b->slots[w.member], last), w.chunk_end[last], vf::kEnsTimeout);
    }
    if (w.done || late) continue;
    while (w.inflight < kInFlight && w.enqueued < w.max_steps)
      if (int rc = wide_enqueue(b, w)) return bfail(b, rc, "wide member launch: " + b->hs[w.member]->err);
  }
  return VF_OK;
}

struct Group {
  int prec;   // 0 double, 1 float
  int variant;
  int csize;
  std::vector<int> members;  // indices into the batch
};

}  // namespace

extern "C" {

int vf_batch_launch(vf_handle* const* hs, int32_t n, const double* t0, const double* endtime, int32_t match_endtime,
                    double maximum_timestep, int64_t max_steps, const vf_batch_options* opt, vf_batch** out) {
  if (!out) return bfail(nullptr, VF_EINVAL, "out is NULL");
  *out = nullptr;
  if (!hs || !t0 || !endtime || n < 1) return bfail(nullptr, VF_EINVAL, "need n >= 1 handles, t0 and endtime");
  const Opts o = resolve(opt);
  const int device = hs[0] ? hs[0]->device : 0;
  for (int i = 0; i < n; ++i) {
    if (!hs[i]) return bfail(nullptr, VF_EINVAL, "NULL handle");
    if (hs[i]->device != device) return bfail(nullptr, VF_EINVAL, "handles live on different devices");
    for (int j = 0; j < i; ++j)
      if (hs[j] == hs[i]) return bfail(nullptr, VF_EINVAL, "a handle appears twice in the batch");
    if (int rc = vf::handle_ready(hs[i])) return bfail(nullptr, rc, std::string("handle not ready: ") + hs[i]->err);
  }
  if (cudaSetDevice(device) != cudaSuccess) return bfail(nullptr, VF_ECUDA, "cudaSetDevice failed");

  vf_batch* b = new (std::nothrow) vf_batch();
  if (!b) return bfail(nullptr, VF_ENOMEM, "host allocation failed");
  b->device = device;
  b->n = n;
  b->hs.assign(hs, hs + n);
  b->collected.assign(n, 0);
  std::string err;
  if (int rc = acquire_slots(n, b->slots, err)) {
    destroy_batch(b);
    return bfail(nullptr, rc, err);
  }
  for (int i = 0; i < n; ++i) std::memset(slot_host(b->slots[i]), 0, sizeof(vf::EnsResult));

  b->start = std::chrono::steady_clock::now();
  b->time_limit_s = o.time_limit_s;
  // Wide members apart; the rest in groups by precision, kernel design and
  // cluster size, largest work first inside a group.
  std::vector<Group> groups;
  std::vector<double> work(n);
  for (int i = 0; i < n; ++i) {
    const vf_handle* h = hs[i];
    if ((long long)h->cfg.nx * h->cfg.ny >= o.wide_cells) {
      Wide w;
      w.member = i;
      w.max_steps = max_steps > 0 ? max_steps : LLONG_MAX;
      w.last_t = t0[i];
      b->wide.push_back(w);
      continue;
    }
    const int prec = h->elem == 8 ? 0 : 1;
    const int var = variant_of(h);
    const int c = fit_cluster(device, (int)h->elem, var, cluster_for(h, o));
    const double dxy = std::min(h->ad.g.dx, h->ad.g.dy);
    work[i] = (double)h->cfg.nx * h->cfg.ny * std::max(0.0, endtime[i] - t0[i]) / dxy;
    auto it = std::find_if(groups.begin(), groups.end(),
                           [&](const Group& g) { return g.prec == prec && g.variant == var && g.csize == c; });
    if (it == groups.end()) {
      groups.push_back(Group{prec, var, c, {}});
      it = groups.end() - 1;
    }
    it->members.push_back(i);
  }
  for (Group& g : groups)
    std::stable_sort(g.members.begin(), g.members.end(), [&](int a, int c) { return work[a] > work[c]; });
  std::stable_sort(groups.begin(), groups.end(), [](const Group& a, const Group& c) { return a.csize > c.csize; });

  // Wide members start first: their first two chunks go in before any cluster.
  for (Wide& w : b->wide) {
    vf_handle* h = hs[w.member];
    bool ok = true;
    for (cudaEvent_t& e : w.ev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    int rc = ok ? vf::handle_begin_loop(h, t0[w.member], endtime[w.member], match_endtime, maximum_timestep)
                : VF_ECUDA;
    for (int k = 0; rc == VF_OK && k < kInFlight && w.enqueued < w.max_steps; ++k) rc = wide_enqueue(b, w);
    if (rc) {
      cudaGetLastError();
      for (Wide& x : b->wide) cudaStreamSynchronize(hs[x.member]->stream);
      const std::string msg = std::string("wide member start: ") + h->err;
      destroy_batch(b);
      return bfail(nullptr, rc ? rc : VF_ECUDA, msg);
    }
  }
  if (groups.empty()) {
    *out = b;
    return VF_OK;
  }

  for (size_t g = 0; g < groups.size(); ++g) {
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      for (Wide& x : b->wide) cudaStreamSynchronize(hs[x.member]->stream);
      destroy_batch(b);
      return bfail(nullptr, VF_ECUDA, "stream creation failed");
    }
    b->streams.push_back(s);
  }
  b->setup = b->streams[0];
  cudaMemPool_t pool = vf::device_pool(device);
  cudaError_t e = pool ? cudaSuccess : cudaErrorMemoryAllocation;
  if (e == cudaSuccess)
    e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&b->epoch_d), sizeof(unsigned long long), pool, b->setup);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->epoch_d, 0, sizeof(unsigned long long), b->setup);
  if (e != cudaSuccess) {
    cudaGetLastError();
    for (Wide& x : b->wide) cudaStreamSynchronize(hs[x.member]->stream);
    destroy_batch(b);
    return bfail(nullptr, VF_ENOMEM, "batch scratch allocation failed");
  }

  // Descriptors: one array per precision, one order array over all groups.
  std::vector<vf::EnsItem<double>> itd;
  std::vector<vf::EnsItem<float>> itf;
  std::vector<int> order;
  std::vector<int> group_base;
  for (const Group& g : groups) {
    group_base.push_back((int)order.size());
    for (int i : g.members) {
      vf_handle* h = hs[i];
      vf::EnsResult* res = slot_dev(b->slots[i]);
      if (g.prec == 0) {
        order.push_back((int)itd.size());
        itd.push_back(make_item<double>(h, h->ad, t0[i], endtime[i], match_endtime, maximum_timestep, max_steps, res,
                                         b->epoch_d));
        itd.back().seg_rows = seg_rows_for(h, g.csize, o.seg_rows);
      } else {
        order.push_back((int)itf.size());
        itf.push_back(make_item<float>(h, h->af, t0[i], endtime[i], match_endtime, maximum_timestep, max_steps, res,
                                        b->epoch_d));
        itf.back().seg_rows = seg_rows_for(h, g.csize, o.seg_rows);
      }
    }
  }

  if (!itd.empty())
    e = cudaMallocFromPoolAsync(&b->items_d[0], sizeof(vf::EnsItem<double>) * itd.size(), pool, b->setup);
  if (e == cudaSuccess && !itf.empty())
    e = cudaMallocFromPoolAsync(&b->items_d[1], sizeof(vf::EnsItem<float>) * itf.size(), pool, b->setup);
  if (e == cudaSuccess) e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&b->order_d), sizeof(int) * order.size(), pool, b->setup);
  if (e == cudaSuccess && !itd.empty())
    e = cudaMemcpyAsync(b->items_d[0], itd.data(), sizeof(vf::EnsItem<double>) * itd.size(), cudaMemcpyHostToDevice,
                        b->setup);
  if (e == cudaSuccess && !itf.empty())
    e = cudaMemcpyAsync(b->items_d[1], itf.data(), sizeof(vf::EnsItem<float>) * itf.size(), cudaMemcpyHostToDevice,
                        b->setup);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->order_d, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice, b->setup);
  // The copies read pageable host vectors: finish them before the vectors go.
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->setup);
  if (e != cudaSuccess) {
    cudaGetLastError();
    for (Wide& x : b->wide) cudaStreamSynchronize(hs[x.member]->stream);
    destroy_batch(b);
    return bfail(nullptr, VF_ECUDA, std::string("batch descriptors: ") + cudaGetErrorString(e));
  }
  const unsigned long long limit_ns = (unsigned long long)(o.time_limit_s * 1e9);
  for (size_t g = 0; g < groups.size(); ++g) {
    const Group& gr = groups[g];
    const int* ord = b->order_d + group_base[g];
    const int cnt = (int)gr.members.size();
    e = gr.prec == 0 ? vf::launch_ensemble(static_cast<const vf::EnsItem<double>*>(b->items_d[0]), ord, cnt,
                                           gr.csize, gr.variant, limit_ns, b->streams[g])
                     : vf::launch_ensemble(static_cast<const vf::EnsItem<float>*>(b->items_d[1]), ord, cnt, gr.csize,
                                           gr.variant, limit_ns, b->streams[g]);
    if (e != cudaSuccess) {
      cudaGetLastError();
      // Launches already issued run to completion before anything is freed.
      for (size_t k = 0; k < g; ++k) cudaStreamSynchronize(b->streams[k]);
      for (Wide& x : b->wide) cudaStreamSynchronize(hs[x.member]->stream);
      destroy_batch(b);
      return bfail(nullptr, VF_ECUDA, std::string("ensemble launch: ") + cudaGetErrorString(e));
    }
    hs[gr.members.front()]->launches += 1;  // one launch for the whole group
  }
  *out = b;
  return VF_OK;
}

int vf_batch_poll(vf_batch* b, int32_t* n_done) {
  if (!b || !n_done) return bfail(b, VF_EINVAL, "NULL argument");
  if (int rc = pump(b)) return rc;
  int c = 0;
  for (int i = 0; i < b->n; ++i) c += slot_done(b->slots[i]) ? 1 : 0;
  *n_done = c;
  return VF_OK;
}

int vf_batch_is_done(vf_batch* b, int32_t i) {
  if (!b || i < 0 || i >= b->n) return bfail(b, VF_EINVAL, "bad batch index");
  if (int rc = pump(b)) return rc;
  return slot_done(b->slots[i]) ? 1 : 0;
}

int vf_batch_collect(vf_batch* b, int32_t i, double* t_out, int64_t* steps_out, double* last_dt_out,
                     int32_t* status_out) {
  if (!b || i < 0 || i >= b->n) return bfail(b, VF_EINVAL, "bad batch index");
  if (!slot_done(b->slots[i])) return bfail(b, VF_ESTATE, "simulation has not finished");
  const vf::EnsResult* r = slot_host(b->slots[i]);
  if (!b->collected[i]) {
    if (r->steps & 1) std::swap(b->hs[i]->U[0], b->hs[i]->U[1]);
    b->collected[i] = 1;
  }
  if (t_out) *t_out = r->t;
  if (steps_out) *steps_out = r->steps;
  if (last_dt_out) *last_dt_out = r->last_dt;
  if (status_out) *status_out = r->status;
  return VF_OK;
}

int vf_batch_wait(vf_batch* b) {
  if (!b) return bfail(b, VF_EINVAL, "NULL batch");
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, VF_ECUDA, "cudaSetDevice failed");
  for (;;) {  // wide members need the host to feed them
    if (int rc = pump(b)) return rc;
    bool all = true;
    for (const Wide& w : b->wide) all = all && w.done;
    if (all) break;
    for (Wide& w : b->wide)
      if (!w.done && w.inflight > 0) {
        cudaEventSynchronize(w.ev[w.head % kInFlight]);
        break;
      }
  }
  for (cudaStream_t s : b->streams) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return bfail(b, VF_ECUDA, std::string("ensemble: ") + cudaGetErrorString(e));
  }
  for (int i = 0; i < b->n; ++i)
    if (!slot_done(b->slots[i])) return bfail(b, VF_ECUDA, "ensemble finished without a result");
  return VF_OK;
}

int vf_batch_free(vf_batch* b) {
  if (!b) return VF_OK;
  int rc = vf_batch_wait(b);
  if (rc == VF_OK)
    for (int i = 0; i < b->n; ++i) vf_batch_collect(b, i, nullptr, nullptr, nullptr, nullptr);
  if (rc != VF_OK) g_batch_error = b->err;
  destroy_batch(b);
  return rc;
}

int vf_batch_simulate(vf_handle* const* hs, int32_t n, const double* t0, const double* endtime, int32_t match_endtime,
                      double maximum_timestep, int64_t max_steps, const vf_batch_options* opt, double* t_out,
                      int64_t* steps_out, double* last_dt_out, int32_t* status_out) {
  vf_batch* b = nullptr;
  int rc = vf_batch_launch(hs, n, t0, endtime, match_endtime, maximum_timestep, max_steps, opt, &b);
  if (rc) return rc;
  rc = vf_batch_wait(b);
  if (rc) {
    g_batch_error = b->err;
    destroy_batch(b);
    return rc;
  }
  for (int i = 0; i < n; ++i) {
    double t = 0, ldt = 0;
    int64_t st = 0;
    int32_t s = 0;
    vf_batch_collect(b, i, &t, &st, &ldt, &s);
    if (t_out) t_out[i] = t;
    if (steps_out) steps_out[i] = st;
    if (last_dt_out) last_dt_out[i] = ldt;
    if (status_out) status_out[i] = s;
  }
  destroy_batch(b);
  return VF_OK;
}

int vf_batch_cluster_size(vf_handle* h, const vf_batch_options* opt, int32_t* csize_out) {
  if (!h || !csize_out) return bfail(nullptr, VF_EINVAL, "NULL argument");
  if (cudaSetDevice(h->device) != cudaSuccess) return bfail(nullptr, VF_ECUDA, "cudaSetDevice failed");
  *csize_out = fit_cluster(h->device, (int)h->elem, variant_of(h), cluster_for(h, resolve(opt)));
  return VF_OK;
}

const char* vf_batch_last_error(vf_batch* b) { return b ? b->err.c_str() : g_batch_error.c_str(); }

}  // extern "C"
