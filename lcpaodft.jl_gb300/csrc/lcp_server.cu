// Serving engine: SCF grid-step requests for many structures, each with its
// orbital tables and step buffers resident on the device (an lcp_job).
//
// Admission: a structure's device footprint (with the tables its precision
// needs) is charged against a byte budget.  A structure that does not fit
// the free budget waits in an admission queue, with its requests, until
// removals free enough of the budget (first come, first admitted); only a
// structure larger than the whole budget is refused.
//
// Continuous batching: each of `nslots` execution slots -- a context of its
// own (stream and workspaces) with a worker thread -- repeatedly takes the
// pending requests of idle admitted structures, oldest first, up to
// `max_batch` of them with one SpinPol and xc, and runs them as ONE batched
// grid step (lcp_batch re-assembled over those jobs: one persistent
// tensor-core launch per contraction over the bricks of every request's
// cell, one FFT solve per grid shape, tiled grid kernels over all cells).
// Requests that arrive while a batch is on the GPU join the next batch of a
// free slot, and the slots' batches overlap on the device.  A batch of one
// (or a server at FP64 / FP32, or "nc" structures) runs the single-job step.
// Latency is measured from submission to the moment the worker sees the
// result on the host.
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

#include "lcp_api_state.h"

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

enum { kAdmitted = 0, kWaiting = 1, kAdmitting = 2 };

struct Structure {
  lcp_job* job = nullptr;
  int nspin = 1;
  int64_t hsize = 0;
  int64_t footprint = 0;  // charged against the budget (an estimate while not admitted)
  int state = kAdmitted;
  bool busy = false;
  int64_t queued = 0;          // requests submitted and not yet completed
  std::vector<double*> free_dm;  // pinned staging buffers
};

}  // namespace

struct lcp_server {
  int device = 0;
  int32_t precision = LCP_PREC_BF16X3;
  int32_t max_batch = 1;  // requests per batched step
  int64_t budget = 0, resident = 0;
  std::vector<lcp_ctx*> slots;
  std::vector<lcp_batch*> runners;  // per slot, re-assembled for every batch
  std::deque<int32_t> waiting;      // structures in the admission queue, in order
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
  int64_t submitted = 0, completed = 0, batches = 0, batched_requests = 0;
  double assemble_ms = 0.0, batch_ms = 0.0;  // host time of the batched steps' assembly, and their wall time
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

  // Whether request r can join `batch` (same SpinPol and xc; the batched
  // step takes split-BF16 "off"/"on" jobs).
  bool joins(const std::vector<Request*>& batch, const Request* r) const {
    if (batch.empty()) return true;
    if (max_batch < 2 || precision != LCP_PREC_BF16X3) return false;
    const lcp_job* a = batch.front()->job;
    const lcp_job* b = r->job;
    return a->spinpol != LCP_SPIN_NC && b->spinpol == a->spinpol && b->xc == a->xc;
  }

  void finish(Request* r) {  // under mu
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

  // The requests of one batched step on this slot: D in, the step, the
  // energies out, one wait.
  lcp_status run_batch(int slot, std::vector<Request*>& batch) {
    lcp_ctx* ctx = slots[slot];
    cudaStream_t st = streams[slot];
    if (!runners[slot]) runners[slot] = batch_new(device);
    std::vector<lcp_job*> jobs;
    for (Request* r : batch) jobs.push_back(r->job);
    const Clock::time_point t0 = Clock::now();
    lcp_status s = batch_assemble(ctx, runners[slot], (int32_t)jobs.size(), jobs.data(), 0);
    const Clock::time_point t1 = Clock::now();
    for (size_t k = 0; k < batch.size() && s == LCP_OK; ++k) {
      Request* r = batch[k];
      for (int c = 0; c < r->nspin && s == LCP_OK; ++c)
        if (cudaMemcpyAsync(r->job->dm[c].p, r->dm + (size_t)c * r->hsize, r->hsize * sizeof(double),
                            cudaMemcpyHostToDevice, st) != cudaSuccess)
          s = LCP_EDEVICE;
    }
    if (s == LCP_OK) s = batch_record(runners[slot], st);
    for (size_t k = 0; k < batch.size() && s == LCP_OK; ++k)
      s = lcp_job_energies_async(ctx, batch[k]->job, batch[k]->energies);
    if (s == LCP_OK) s = batch_status(runners[slot], st);  // waits for the stream
    const Clock::time_point t2 = Clock::now();
    {
      std::lock_guard<std::mutex> lk(mu);
      assemble_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
      batch_ms += std::chrono::duration<double, std::milli>(t2 - t0).count();
    }
    return s;
  }

  // One worker per slot: take the pending requests of idle admitted
  // structures (oldest first, up to max_batch that batch together), run
  // them on this slot, wait, publish the results.
  void run(int slot) {
    cudaSetDevice(device);
    while (true) {
      std::vector<Request*> batch;
      {
        std::unique_lock<std::mutex> lk(mu);
        while (true) {
          for (auto it = pending.begin(); it != pending.end() && (int)batch.size() < std::max(1, max_batch);) {
            Structure& st = structs[(*it)->id];
            if (!st.busy && st.state == kAdmitted && joins(batch, *it)) {
              st.busy = true;
              batch.push_back(*it);
              it = pending.erase(it);
            } else {
              ++it;
            }
          }
          if (!batch.empty() || stop) break;
          cv_work.wait_for(lk, std::chrono::milliseconds(5));
        }
        if (batch.size() > 1) {
          batches++;
          batched_requests += (int64_t)batch.size();
        }
      }
      if (batch.empty()) break;  // stopping, nothing runnable
      if (batch.size() == 1) {
        Request* r = batch.front();
        r->slot = slot;
        launch(r);
        if (r->status == LCP_OK) {
          const cudaError_t e = cudaEventSynchronize(r->done);
          if (e != cudaSuccess) r->status = LCP_EDEVICE;
        }
        if (r->status == LCP_OK) r->status = lcp_ctx_check_status(slots[slot]);
      } else {
        const lcp_status s = run_batch(slot, batch);
        for (Request* r : batch) {
          r->slot = slot;
          r->status = s;
        }
      }
      const Clock::time_point now = Clock::now();
      {
        std::lock_guard<std::mutex> lk(mu);
        for (Request* r : batch) {
          r->t_done = now;
          finish(r);
        }
      }
      cv_done.notify_all();
      cv_work.notify_all();  // these structures may have more requests waiting
    }
  }

  // Admits queued structures, in order, while they fit the free budget: their
  // precision's tables are built on the admission context (caller's thread).
  lcp_status admit_waiting() {
    std::vector<int32_t> ids;
    {
      std::lock_guard<std::mutex> lk(mu);
      while (!waiting.empty()) {
        Structure& st = structs[waiting.front()];
        if (resident + st.footprint > budget) break;
        resident += st.footprint;
        st.state = kAdmitting;
        ids.push_back(waiting.front());
        waiting.pop_front();
      }
    }
    lcp_status first = LCP_OK;
    for (int32_t id : ids) {
      lcp_job* job = nullptr;
      {
        std::lock_guard<std::mutex> lk(mu);
        job = structs[id].job;
      }
      lcp_status s = lcp_job_prepare(admin, job);
      int64_t fp = 0;
      if (s == LCP_OK) s = lcp_job_footprint(job, &fp);
      {
        std::lock_guard<std::mutex> lk(mu);
        Structure& st = structs[id];
        if (s == LCP_OK) {
          resident += fp - st.footprint;
          st.footprint = fp;
        }
        st.state = kAdmitted;  // a failure shows up in the structure's requests
      }
      if (s != LCP_OK && first == LCP_OK) first = s;
    }
    if (!ids.empty()) cv_work.notify_all();
    return first;
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
  s->precision = precision;
  s->max_batch = precision == LCP_PREC_BF16X3 ? 16 : 1;
  if (cudaSetDevice(device) != cudaSuccess) return fail(LCP_EDEVICE, "cudaSetDevice failed");
  for (int k = 0; k < nslots; ++k) {
    lcp_ctx* c = nullptr;
    lcp_status st = lcp_ctx_create(device, &c);
    if (st) return st;
    s->slots.push_back(c);
    s->runners.push_back(nullptr);
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
  for (auto* r : srv->pending) {  // requests of structures that never ran (the admission queue)
    if (r->done) cudaEventDestroy(r->done);
    if (r->dm) cudaFreeHost(r->dm);
    delete r;
  }
  for (auto* b : srv->runners) lcp_batch_destroy(b);
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
  const int64_t est = job_footprint_estimate(job, srv->precision);
  if (est < 0) return fail(LCP_EINVAL, "the structure's footprint cannot be estimated (bricks)");
  if (est > srv->budget)
    return fail(LCP_ENOMEM, "admission: the structure needs " + std::to_string(est) +
                                " device bytes, more than the whole budget of " + std::to_string(srv->budget));
  bool now = false;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    Structure st;
    st.job = job;
    st.nspin = nspin;
    st.hsize = hsize;
    st.footprint = est;
    now = srv->waiting.empty() && srv->resident + est <= srv->budget;
    st.state = now ? kAdmitting : kWaiting;
    *id = srv->next_id++;
    if (now) srv->resident += est;
    else srv->waiting.push_back(*id);
    srv->structs.emplace(*id, std::move(st));
  }
  if (!now) return LCP_OK;  // admitted when removals free the budget
  // the precision's tables are built now, and the footprint measured
  lcp_status s = lcp_job_prepare(srv->admin, job);
  int64_t fp = 0;
  if (s == LCP_OK) s = lcp_job_footprint(job, &fp);
  std::lock_guard<std::mutex> lk(srv->mu);
  Structure& st = srv->structs[*id];
  if (s != LCP_OK) {
    srv->resident -= st.footprint;
    srv->structs.erase(*id);
    return s;
  }
  srv->resident += fp - st.footprint;
  st.footprint = fp;
  st.state = kAdmitted;
  return LCP_OK;
}

lcp_status lcp_server_remove(lcp_server* srv, int32_t id) {
  if (!srv) return fail(LCP_EINVAL, "NULL server");
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->structs.find(id);
    if (it == srv->structs.end()) return fail(LCP_EINVAL, "unknown structure id");
    if (it->second.queued > 0) return fail(LCP_ESTATE, "the structure has requests in flight");
    if (it->second.state == kAdmitting) return fail(LCP_ESTATE, "the structure is being admitted");
    for (double* p : it->second.free_dm) cudaFreeHost(p);
    if (it->second.state == kWaiting) {
      for (auto w = srv->waiting.begin(); w != srv->waiting.end(); ++w)
        if (*w == id) {
          srv->waiting.erase(w);
          break;
        }
    } else {
      srv->resident -= it->second.footprint;
    }
    srv->structs.erase(it);
  }
  return srv->admit_waiting();
}

// 0: admitted, 1: waiting in the admission queue, 2: being admitted.
lcp_status lcp_server_state(lcp_server* srv, int32_t id, int32_t* state) {
  if (!srv || !state) return fail(LCP_EINVAL, "NULL argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  auto it = srv->structs.find(id);
  if (it == srv->structs.end()) return fail(LCP_EINVAL, "unknown structure id");
  *state = it->second.state;
  return LCP_OK;
}

lcp_status lcp_server_set_max_batch(lcp_server* srv, int32_t max_batch) {
  if (!srv) return fail(LCP_EINVAL, "NULL server");
  if (max_batch < 1 || max_batch > 4096) return fail(LCP_EINVAL, "max_batch must be in 1..4096");
  if (max_batch > 1 && srv->precision != LCP_PREC_BF16X3)
    return fail(LCP_ENOTSUP, "batched serving steps run the split-BF16 contractions (precision bf16x3)");
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->max_batch = max_batch;
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

lcp_status lcp_server_batch_stats(lcp_server* srv, int64_t* out5) {
  if (!srv || !out5) return fail(LCP_EINVAL, "NULL argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  out5[0] = srv->batches;
  out5[1] = srv->batched_requests;
  out5[2] = (int64_t)srv->waiting.size();
  out5[3] = (int64_t)(srv->assemble_ms * 1000.0);
  out5[4] = (int64_t)(srv->batch_ms * 1000.0);
  return LCP_OK;
}

}  // extern "C"
