// vf_server.cu -- the serving engine (vf_server_*) of include/volumefluxes_sm103.h.
//
// Requests are whole flood simulations: a configuration, a bottom, an initial
// interior state and an end time, with output buffers for the final state.
// An engine thread runs, in a loop:
//   1. completion: every running request whose done flag is set (the batch's
//      pinned, mapped result slot) is collected, its final interior state is
//      copied to the caller's buffers, its handle is destroyed and its device
//      bytes return to the budget;
//   2. admission: queued requests, oldest first, get a handle (device memory
//      from the library pool), their bottom and state are uploaded, and their
//      bytes are charged, for as long as the HBM budget holds;
//   3. launch: everything admitted in this round starts as one batch
//      (vf_batch_launch) on its own streams, while earlier batches keep
//      running: continuous batching, with the GPU's block scheduler sharing the
//      SMs between the batches in flight.
// A request's result does not depend on what runs beside it: each simulation
// is one cluster (or one whole-grid kernel stream) with its own dt and data.
//
// The loop also feeds the wide members of running batches, about every 100 us
// while anything runs (it sleeps otherwise), so the GPU never waits for the
// caller; the caller's submit/poll/result calls only take the engine's lock.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "vf_handle.h"

namespace {

enum class ReqState { kQueued, kRunning, kDone, kFailed };

struct Request {
  vf_config cfg;
  const void* B = nullptr;
  const void* w = nullptr;
  const void* hu = nullptr;
  const void* hv = nullptr;
  void* ow = nullptr;
  void* ohu = nullptr;
  void* ohv = nullptr;
  double t0 = 0, endtime = 0;
  size_t bytes = 0;
  ReqState state = ReqState::kQueued;
  vf_handle* h = nullptr;
  int batch = -1;  // index into the server's batch table
  int slot = -1;   // index inside that batch
  double t = 0, last_dt = 0;
  int64_t steps = 0;
  int32_t status = 0;
  int error = 0;
  std::string message;
  bool reported = false;
  double submit_s = 0, admit_s = 0, done_s = 0;  // seconds since the server started
};

struct Batch {
  vf_batch* b = nullptr;
  int remaining = 0;
};

}  // namespace

struct vf_server {
  int device = 0;
  size_t budget = 0, used = 0;
  vf_batch_options opt{};
  bool has_opt = false;
  int64_t max_steps = 0;
  int64_t next_ticket = 1;
  std::deque<int64_t> queue;
  std::map<int64_t, Request> reqs;
  std::vector<Batch> batches;
  int64_t launches = 0;
  std::string err;        // last caller-side error
  std::string engine_err; // last engine error (reported by the next poll)
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv;
  std::thread engine;
  bool stop = false;
};

namespace {

thread_local std::string g_server_error;

int sfail(vf_server* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  else g_server_error = msg;
  return code;
}

double now_s(const vf_server* s) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->t0).count();
}

void finish_request(vf_server* s, Request& r, int error, const std::string& msg) {
  r.done_s = now_s(s);
  if (r.h) {
    vf_destroy(r.h);
    r.h = nullptr;
    s->used -= r.bytes;
  }
  r.error = error;
  r.message = msg;
  r.state = error ? ReqState::kFailed : ReqState::kDone;
}

// Handle with bottom and state uploaded; on failure the request fails.
bool admit(vf_server* s, Request& r) {
  vf_handle* h = nullptr;
  vf_config c = r.cfg;
  c.device = s->device;
  int rc = vf_create(&c, &h);
  if (rc) {
    finish_request(s, r, rc, vf_last_error(nullptr));
    return false;
  }
  r.h = h;
  s->used += r.bytes;
  if (!c.bottom_is_constant && (rc = vf_upload_bottom(h, r.B))) {
    finish_request(s, r, rc, vf_last_error(h));
    return false;
  }
  if ((rc = vf_set_interior_state(h, r.w, r.hu, r.hv))) {
    finish_request(s, r, rc, vf_last_error(h));
    return false;
  }
  return true;
}

void complete(vf_server* s) {
  for (auto& kv : s->reqs) {
    Request& r = kv.second;
    if (r.state != ReqState::kRunning) continue;
    Batch& bt = s->batches[r.batch];
    if (vf_batch_is_done(bt.b, r.slot) != 1) continue;
    double t = 0, ldt = 0;
    int64_t st = 0;
    int32_t status = 0;
    int rc = vf_batch_collect(bt.b, r.slot, &t, &st, &ldt, &status);
    if (rc == VF_OK) rc = vf_get_interior_state(r.h, r.ow, r.ohu, r.ohv);
    r.t = t;
    r.steps = st;
    r.last_dt = ldt;
    r.status = status;
    finish_request(s, r, rc, rc ? std::string(vf_last_error(r.h)) : std::string());
    if (--bt.remaining == 0) {
      vf_batch_free(bt.b);
      bt.b = nullptr;
    }
  }
}

int admit_and_launch(vf_server* s) {
  std::vector<vf_handle*> hs;
  std::vector<double> t0, ends;
  std::vector<int64_t> tickets;
  while (!s->queue.empty()) {
    const int64_t tk = s->queue.front();
    Request& r = s->reqs[tk];
    if (s->used + r.bytes > s->budget) break;  // oldest first: wait for memory
    s->queue.pop_front();
    r.admit_s = now_s(s);
    if (!admit(s, r)) continue;
    hs.push_back(r.h);
    t0.push_back(r.t0);
    ends.push_back(r.endtime);
    tickets.push_back(tk);
  }
  if (hs.empty()) return VF_OK;
  vf_batch* b = nullptr;
  int rc = vf_batch_launch(hs.data(), (int32_t)hs.size(), t0.data(), ends.data(), 1, -1.0, s->max_steps,
                           s->has_opt ? &s->opt : nullptr, &b);
  if (rc) {
    const std::string msg = vf_batch_last_error(nullptr);
    for (int64_t tk : tickets) finish_request(s, s->reqs[tk], rc, msg);
    s->engine_err = "batch launch: " + msg;
    return rc;
  }
  s->batches.push_back(Batch{b, (int)hs.size()});
  s->launches += 1;
  const int bi = (int)s->batches.size() - 1;
  for (size_t i = 0; i < tickets.size(); ++i) {
    Request& r = s->reqs[tickets[i]];
    r.state = ReqState::kRunning;
    r.batch = bi;
    r.slot = (int)i;
  }
  return VF_OK;
}

bool busy(const vf_server* s) {
  if (!s->queue.empty()) return true;
  for (const auto& kv : s->reqs)
    if (kv.second.state == ReqState::kRunning) return true;
  return false;
}

// The engine thread: complete, admit, launch, feed wide members; about every
// 100 us while anything runs, asleep otherwise.
void engine_loop(vf_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    complete(s);
    admit_and_launch(s);
    for (Batch& bt : s->batches) {
      int32_t nd = 0;
      if (bt.b) vf_batch_poll(bt.b, &nd);  // retires and refills wide members' chunks
    }
    if (busy(s)) {
      s->cv.wait_for(lk, std::chrono::microseconds(100));
    } else {
      s->cv.wait(lk, [s] { return s->stop || !s->queue.empty(); });
    }
  }
}

}  // namespace

extern "C" {

int vf_server_create(int32_t device, int64_t hbm_budget_bytes, const vf_batch_options* opt, int64_t max_steps,
                     vf_server** out) {
  if (!out) return sfail(nullptr, VF_EINVAL, "out is NULL");
  *out = nullptr;
  if (hbm_budget_bytes <= 0) return sfail(nullptr, VF_EINVAL, "the HBM budget must be positive");
  vf_server* s = new (std::nothrow) vf_server();
  if (!s) return sfail(nullptr, VF_ENOMEM, "host allocation failed");
  s->device = device;
  s->budget = (size_t)hbm_budget_bytes;
  s->max_steps = max_steps;
  if (opt) {
    s->opt = *opt;
    s->has_opt = true;
  }
  s->t0 = std::chrono::steady_clock::now();
  try {
    s->engine = std::thread(engine_loop, s);
  } catch (...) {
    delete s;
    return sfail(nullptr, VF_ENOMEM, "engine thread could not start");
  }
  *out = s;
  return VF_OK;
}

int vf_server_submit(vf_server* s, const vf_config* cfg, const void* B_corners, const void* w, const void* hu,
                     const void* hv, double t0, double endtime, void* out_w, void* out_hu, void* out_hv,
                     int64_t* ticket_out) {
  if (!s || !cfg || !w || !hu || !hv || !ticket_out) return sfail(s, VF_EINVAL, "NULL argument");
  if (!cfg->bottom_is_constant && !B_corners) return sfail(s, VF_EINVAL, "bottom corners missing");
  for (int i = 0; i < cfg->n_sources && i < VF_MAX_SOURCES; ++i) {
    const int k = cfg->source_kind[i];
    if (k != VF_SRC_BOTTOM && k != VF_SRC_CONST_RAIN && k != VF_SRC_CONST_INFIL)
      return sfail(s, VF_EINVAL, "served requests take SourceTermBottom, ConstantRain and ConstantInfiltration only");
  }
  Request r;
  r.cfg = *cfg;
  r.B = B_corners;
  r.w = w;
  r.hu = hu;
  r.hv = hv;
  r.ow = out_w;
  r.ohu = out_hu;
  r.ohv = out_hv;
  r.t0 = t0;
  r.endtime = endtime;
  r.bytes = vf::handle_device_bytes(cfg);
  if (r.bytes > s->budget) return sfail(s, VF_ENOMEM, "request larger than the whole HBM budget");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r.submit_s = now_s(s);
    const int64_t tk = s->next_ticket++;
    s->reqs.emplace(tk, r);
    s->queue.push_back(tk);
    *ticket_out = tk;
  }
  s->cv.notify_one();
  return VF_OK;
}

int vf_server_poll(vf_server* s, int64_t* done_tickets, int32_t capacity, int32_t* n_done) {
  if (!s) return sfail(s, VF_EINVAL, "NULL server");
  std::lock_guard<std::mutex> lk(s->mu);
  int32_t n = 0;
  for (auto& kv : s->reqs) {
    Request& r = kv.second;
    if ((r.state == ReqState::kDone || r.state == ReqState::kFailed) && !r.reported && n < capacity) {
      if (done_tickets) done_tickets[n] = kv.first;
      r.reported = true;
      ++n;
    }
  }
  if (n_done) *n_done = n;
  if (!s->engine_err.empty()) {
    s->err = s->engine_err;
    s->engine_err.clear();
    return VF_ECUDA;
  }
  return VF_OK;
}

int vf_server_result(vf_server* s, int64_t ticket, double* t_out, int64_t* steps_out, double* last_dt_out,
                     int32_t* status_out) {
  if (!s) return sfail(s, VF_EINVAL, "NULL server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(s, VF_EINVAL, "unknown ticket");
  const Request& r = it->second;
  if (r.state == ReqState::kQueued || r.state == ReqState::kRunning) return sfail(s, VF_ESTATE, "request not finished");
  if (t_out) *t_out = r.t;
  if (steps_out) *steps_out = r.steps;
  if (last_dt_out) *last_dt_out = r.last_dt;
  if (status_out) *status_out = r.status;
  if (r.state == ReqState::kFailed) return sfail(s, r.error, r.message);
  return VF_OK;
}

int vf_server_timing(vf_server* s, int64_t ticket, double* submit_s, double* admit_s, double* done_s) {
  if (!s) return sfail(s, VF_EINVAL, "NULL server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(s, VF_EINVAL, "unknown ticket");
  if (submit_s) *submit_s = it->second.submit_s;
  if (admit_s) *admit_s = it->second.admit_s;
  if (done_s) *done_s = it->second.done_s;
  return VF_OK;
}

int vf_server_release(vf_server* s, int64_t ticket) {
  if (!s) return sfail(s, VF_EINVAL, "NULL server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(s, VF_EINVAL, "unknown ticket");
  if (it->second.state == ReqState::kQueued || it->second.state == ReqState::kRunning)
    return sfail(s, VF_ESTATE, "request not finished");
  s->reqs.erase(it);
  return VF_OK;
}

int vf_server_stats(vf_server* s, int64_t* used_bytes, int32_t* queued, int32_t* running, int64_t* launches) {
  if (!s) return sfail(s, VF_EINVAL, "NULL server");
  std::lock_guard<std::mutex> lk(s->mu);
  int32_t q = 0, r = 0;
  for (auto& kv : s->reqs) {
    q += kv.second.state == ReqState::kQueued;
    r += kv.second.state == ReqState::kRunning;
  }
  if (used_bytes) *used_bytes = (int64_t)s->used;
  if (queued) *queued = q;
  if (running) *running = r;
  if (launches) *launches = s->launches;
  return VF_OK;
}

int vf_server_destroy(vf_server* s) {
  if (!s) return VF_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_one();
  if (s->engine.joinable()) s->engine.join();
  cudaSetDevice(s->device);
  for (Batch& bt : s->batches)
    if (bt.b) vf_batch_free(bt.b);
  for (auto& kv : s->reqs)
    if (kv.second.h) vf_destroy(kv.second.h);
  delete s;
  return VF_OK;
}

const char* vf_server_last_error(vf_server* s) { return s ? s->err.c_str() : g_server_error.c_str(); }

}  // extern "C"
