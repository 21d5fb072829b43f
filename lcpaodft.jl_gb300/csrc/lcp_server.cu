// Serving engine: SCF grid-step requests for many structures, each with its
// orbital tables and step buffers resident on the device (an lcp_job).
//
// Structures are admitted by HBM footprint against a budget.  Requests carry
// a new density matrix.  Each of `nslots` execution slots -- a context of its
// own (stream and workspaces) with a worker thread -- takes the oldest pending
// request whose structure is idle, so requests on different slots run
// concurrently on the device, kernel launches are issued from several host
// threads, and new requests start while others are still in flight.  Latency
// is measured from submission to the moment the slot's worker sees the result
// (its completion event).
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "lcp_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t tag = 0;
  int32_t id = -1;
  lcp_job* job = nullptr;  // copied from the structure at submission: the
  int nspin = 1;           // worker never reads the structure map unlocked
  int64_t hsize = 0;
  int slot = -1;
  double* dm = nullptr;       // pinned, nspin * hsize
  double* energies = nullptr; // pinned, 5 (inside the server's energy arena)
  cudaEvent_t done = nullptr;
  Clock::time_point t_submit, t_done;
  lcp_status status = LCP_OK;
};

struct Structure {
  lcp_job* job = nullptr;
  int nspin = 1;
  int64_t hsize = 0;
  int64_t footprint = 0;
  bool busy = false;
  int64_t queued = 0;          // requests submitted and not yet completed
  std::vector<double*> free_dm;  // pinned staging buffers
};

lcp_status fail(lcp_status code, const std::string& msg) {
  lcp::set_error(msg);
  return code;
}

}  // namespace

struct lcp_server {
  int device = 0;
  int64_t budget = 0, resident = 0;
  std::vector<lcp_ctx*> slots;
  lcp_ctx* admin = nullptr;  // prepares structures' tables at admission (caller's thread)
  std::vector<cudaStream_t> streams;
  std::map<int32_t, Structure> structs;
  int32_t next_id = 0;
  double* energy_arena = nullptr;  // pinned, 8 doubles per entry
  std::vector<double*> free_energy;
  std::deque<Request*> pending;
  std::deque<Request*> done;
  std::vector<cudaEvent_t> free_events;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::vector<std::thread> workers;
  int64_t submitted = 0, completed = 0;
  lcp_status sticky = LCP_OK;
  std::string sticky_msg;

  void launch(Request* r) {
    lcp_ctx* ctx = slots[r->slot];
    const double* dm[4];
    for (int c = 0; c < r->nspin; ++c) dm[c] = r->dm + (size_t)c * r->hsize;
    lcp_status s = lcp_job_set_dm(ctx, r->job, dm);
    if (s == LCP_OK) s = lcp_job_step(ctx, r->job);
    if (s == LCP_OK) s = lcp_job_energies_async(ctx, r->job, r->energies);
    if (s == LCP_OK && cudaEventRecord(r->done, streams[r->slot]) != cudaSuccess) s = LCP_EDEVICE;
    r->status = s;
  }

  // One worker per slot: take the oldest pending request whose structure is
  // idle, run it on this slot, wait for it, publish the result.
  void run(int slot) {
    cudaSetDevice(device);
    while (true) {
      Request* r = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        while (true) {
          for (auto it = pending.begin(); it != pending.end(); ++it) {
            Structure& st = structs[(*it)->id];
            if (!st.busy) {
              st.busy = true;
              r = *it;
              pending.erase(it);
              break;
            }
          }
          if (r || (stop && pending.empty())) break;
          cv_work.wait_for(lk, std::chrono::milliseconds(5));
        }
      }
      if (!r) break;
      r->slot = slot;
      launch(r);
      if (r->status == LCP_OK) {
        const cudaError_t e = cudaEventSynchronize(r->done);
        if (e != cudaSuccess) r->status = LCP_EDEVICE;
      }
      if (r->status == LCP_OK) r->status = lcp_ctx_check_status(slots[slot]);
      r->t_done = Clock::now();
      {
        std::lock_guard<std::mutex> lk(mu);
        Structure& st = structs[r->id];
        st.busy = false;
        st.queued--;
        st.free_dm.push_back(r->dm);
        r->dm = nullptr;
        if (r->status != LCP_OK && sticky == LCP_OK) {
          sticky = r->status;
          sticky_msg = lcp_last_error() ? lcp_last_error() : "request failed";
        }
        done.push_back(r);
        completed++;
      }
      cv_done.notify_all();
      cv_work.notify_all();  // this structure may have more requests waiting
    }
  }
};

extern "C" {

lcp_status lcp_server_create(int32_t device, int32_t nslots, int32_t precision, int64_t budget_bytes,
                             lcp_server** out) {
  if (!out) return fail(LCP_EINVAL, "NULL argument");
  *out = nullptr;
  if (nslots < 1 || nslots > 64) return fail(LCP_EINVAL, "nslots must be in 1..64");
  if (budget_bytes <= 0) return fail(LCP_EINVAL, "budget must be positive");
  std::unique_ptr<lcp_server> s(new lcp_server());
  s->device = device;
  s->budget = budget_bytes;
  if (cudaSetDevice(device) != cudaSuccess) return fail(LCP_EDEVICE, "cudaSetDevice failed");
  for (int k = 0; k < nslots; ++k) {
    lcp_ctx* c = nullptr;
    lcp_status st = lcp_ctx_create(device, &c);
    if (st) return st;
    s->slots.push_back(c);
    cudaStream_t stream;
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess)
      return fail(LCP_EDEVICE, "cudaStreamCreate failed");
    s->streams.push_back(stream);
    if ((st = lcp_ctx_set_stream(c, stream))) return st;
    if ((st = lcp_ctx_set_precision(c, precision))) return st;
  }
  {
    lcp_status st = lcp_ctx_create(device, &s->admin);
    if (st) return st;
    if ((st = lcp_ctx_set_precision(s->admin, precision))) return st;
  }
  constexpr int kEnergySlots = 16384;
  if (cudaHostAlloc(&s->energy_arena, (size_t)kEnergySlots * 8 * sizeof(double), cudaHostAllocDefault) != cudaSuccess)
    return fail(LCP_ENOMEM, "pinned allocation failed");
  for (int k = 0; k < kEnergySlots; ++k) s->free_energy.push_back(s->energy_arena + (size_t)k * 8);
  lcp_server* raw = s.get();
  for (int k = 0; k < nslots; ++k) s->workers.emplace_back([raw, k]() { raw->run(k); });
  *out = s.release();
  return LCP_OK;
}

void lcp_server_destroy(lcp_server* srv) {
  if (!srv) return;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  for (auto& w : srv->workers)
    if (w.joinable()) w.join();
  cudaSetDevice(srv->device);
  for (auto* r : srv->done) {
    if (r->done) cudaEventDestroy(r->done);
    delete r;
  }
  for (auto e : srv->free_events) cudaEventDestroy(e);
  for (auto& kv : srv->structs)
    for (double* p : kv.second.free_dm) cudaFreeHost(p);
  if (srv->energy_arena) cudaFreeHost(srv->energy_arena);
  for (auto* c : srv->slots) lcp_ctx_destroy(c);
  if (srv->admin) lcp_ctx_destroy(srv->admin);
  for (auto st : srv->streams) cudaStreamDestroy(st);
  delete srv;
}

lcp_status lcp_server_add(lcp_server* srv, lcp_job* job, int32_t nspin, int64_t hsize, int32_t* id) {
  if (!srv || !job || !id) return fail(LCP_EINVAL, "NULL argument");
  if (nspin < 1 || nspin > 4 || hsize < 0) return fail(LCP_EINVAL, "bad nspin / hsize");
  // the precision's tables are built now, so that the footprint is complete
  lcp_status s = lcp_job_prepare(srv->admin, job);
  if (s) return s;
  int64_t fp = 0;
  if ((s = lcp_job_footprint(job, &fp))) return s;
  std::lock_guard<std::mutex> lk(srv->mu);
  if (srv->resident + fp > srv->budget)
    return fail(LCP_ENOMEM, "admission: the structure needs " + std::to_string(fp) + " device bytes; " +
                                std::to_string(srv->budget - srv->resident) + " of the budget are free");
  Structure st;
  st.job = job;
  st.nspin = nspin;
  st.hsize = hsize;
  st.footprint = fp;
  *id = srv->next_id++;
  srv->structs.emplace(*id, std::move(st));
  srv->resident += fp;
  return LCP_OK;
}

lcp_status lcp_server_remove(lcp_server* srv, int32_t id) {
  if (!srv) return fail(LCP_EINVAL, "NULL server");
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->structs.find(id);
  if (it == srv->structs.end()) return fail(LCP_EINVAL, "unknown structure id");
  if (it->second.queued > 0) return fail(LCP_ESTATE, "the structure has requests in flight");
  for (double* p : it->second.free_dm) cudaFreeHost(p);
  srv->resident -= it->second.footprint;
  srv->structs.erase(it);
  return LCP_OK;
}

lcp_status lcp_server_submit(lcp_server* srv, int32_t id, const double* const* dm, uint64_t tag) {
  if (!srv || !dm) return fail(LCP_EINVAL, "NULL argument");
  std::unique_ptr<Request> r(new Request());
  r->tag = tag;
  r->id = id;
  r->t_submit = Clock::now();
  double* buf = nullptr;
  int nspin = 0;
  int64_t hs = 0;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->structs.find(id);
    if (it == srv->structs.end()) return fail(LCP_EINVAL, "unknown structure id");
    nspin = it->second.nspin;
    hs = it->second.hsize;
    r->job = it->second.job;
    r->nspin = nspin;
    r->hsize = hs;
    if (!it->second.free_dm.empty()) {
      buf = it->second.free_dm.back();
      it->second.free_dm.pop_back();
    }
    if (srv->free_energy.empty()) return fail(LCP_ENOMEM, "too many requests outstanding");
    r->energies = srv->free_energy.back();
    srv->free_energy.pop_back();
    if (!srv->free_events.empty()) {
      r->done = srv->free_events.back();
      srv->free_events.pop_back();
    }
  }
  if (!buf && cudaHostAlloc(&buf, (size_t)nspin * hs * sizeof(double) + 8, cudaHostAllocDefault) != cudaSuccess)
    return fail(LCP_ENOMEM, "pinned allocation failed");
  if (!r->done && cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming) != cudaSuccess)
    return fail(LCP_EDEVICE, "cudaEventCreate failed");
  for (int c = 0; c < nspin; ++c) {
    if (!dm[c]) return fail(LCP_EINVAL, "NULL channel");
    std::memcpy(buf + (size_t)c * hs, dm[c], (size_t)hs * sizeof(double));
  }
  r->dm = buf;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->structs[id].queued++;
    srv->pending.push_back(r.release());
    srv->submitted++;
  }
  srv->cv_work.notify_one();
  return LCP_OK;
}

lcp_status lcp_server_poll(lcp_server* srv, int32_t max, int32_t wait_ms, uint64_t* tags, double* energies,
                           double* latency_ms, int32_t* n) {
  if (!srv || !n || (max > 0 && (!tags || !energies || !latency_ms))) return fail(LCP_EINVAL, "NULL argument");
  *n = 0;
  std::unique_lock<std::mutex> lk(srv->mu);
  if (srv->done.empty() && wait_ms > 0)
    srv->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [srv]() { return !srv->done.empty(); });
  while (*n < max && !srv->done.empty()) {
    Request* r = srv->done.front();
    srv->done.pop_front();
    tags[*n] = r->tag;
    for (int k = 0; k < 5; ++k) energies[5 * *n + k] = r->status == LCP_OK ? r->energies[k] : 0.0;
    latency_ms[*n] = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    srv->free_energy.push_back(r->energies);
    srv->free_events.push_back(r->done);
    delete r;
    ++*n;
  }
  if (srv->sticky != LCP_OK) {
    lcp_status s = srv->sticky;
    srv->sticky = LCP_OK;
    return fail(s, "a request failed: " + srv->sticky_msg);
  }
  return LCP_OK;
}

lcp_status lcp_server_stats(lcp_server* srv, int64_t* out4) {
  if (!srv || !out4) return fail(LCP_EINVAL, "NULL argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  out4[0] = srv->submitted;
  out4[1] = srv->completed;
  out4[2] = srv->resident;
  out4[3] = srv->budget;
  return LCP_OK;
}

}  // extern "C"
