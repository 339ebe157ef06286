// Request server: continuous batching of independent simulations on one GPU.
//
// The reference runs a batch either one simulation at a time (run_batch,
// src/Batch.jl:103-145) or in fixed waves sized from a memory plan
// (run_batch_concurrent / plan_batch, src/Batch.jl:21-66,170-263; estimate_memory,
// src/Memory.jl:120-251).  Here requests arrive at any time:
//
//   * an admission thread takes submitted requests in FIFO order while the
//     device-memory budget and the resident-slot count allow, and prepares
//     them (allocation, classification, uploads) while other requests step;
//   * a stepping thread keeps every resident request's stream fed with
//     quanta of steps (two quanta in flight per request), so the kernels of
//     different requests overlap on the GPU, and retires a request as soon as
//     its last quantum has finished; its slot and budget are then free for the
//     next admission.
//
// A request's results stay on its kh_sim until kh_server_release, which frees
// its device memory and returns its bytes to the budget.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/khronos_gb300.h"
#include "kh_simbase.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t ticket = 0;
  kh_sim* sim = nullptr;
  int64_t nsteps = 0;
  int64_t issued = 0;  // steps handed to the GPU
  int64_t est_bytes = 0;
  int32_t state = KH_REQ_QUEUED;
  kh_status status = KH_OK;
  std::string error;
  double t_submit = -1, t_admit = -1, t_start = -1, t_done = -1;
  // stepping thread only
  int slot = -1;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int head = 0, inflight = 0;
};

}  // namespace

struct kh_server {
  kh_server_desc desc{};
  int device = 0;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_admit, cv_step, cv_done;
  std::deque<Request*> pending;  // submitted, not admitted
  std::deque<Request*> ready;    // prepared, waiting for the stepping thread
  std::map<int64_t, std::unique_ptr<Request>> reqs;
  std::deque<int64_t> done_q;  // finished requests not yet reported by wait_any
  int64_t next_ticket = 1;
  int64_t budget_used = 0;  // bytes of admitted, unreleased requests
  int resident = 0;         // admitted and not finished
  std::atomic<bool> stop{false};
  std::vector<cudaStream_t> streams;
  std::vector<int> free_slots;
  std::thread admit_thr, step_thr;
  std::string err;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  bool can_admit_front() const {
    if (pending.empty() || resident >= desc.max_resident) return false;
    return budget_used + pending.front()->est_bytes <= desc.budget_bytes;
  }

  void finish(Request* r, kh_status st, const std::string& msg) {
    // caller holds mu
    r->status = st;
    r->error = msg;
    r->state = st == KH_OK ? KH_REQ_DONE : KH_REQ_FAILED;
    r->t_done = now();
    done_q.push_back(r->ticket);
    --resident;
    cv_done.notify_all();
    cv_admit.notify_all();
  }

  void admit_loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      cv_admit.wait(lk, [&] { return stop || can_admit_front(); });
      if (stop) return;
      Request* r = pending.front();
      pending.pop_front();
      budget_used += r->est_bytes;
      ++resident;
      r->state = KH_REQ_ADMITTED;
      lk.unlock();
      const kh_status st = r->sim->impl->prepare();
      const int64_t actual = r->sim->impl->device_bytes();
      lk.lock();
      // account what prepare() really allocated
      budget_used += actual - r->est_bytes;
      r->est_bytes = actual;
      r->t_admit = now();
      if (st != KH_OK) {
        finish(r, st, r->sim->impl->err);
        continue;
      }
      ready.push_back(r);
      cv_step.notify_all();
    }
  }

  void step_loop() {
    cudaSetDevice(device);
    std::vector<Request*> running;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu);
        if (running.empty()) cv_step.wait(lk, [&] { return stop || !ready.empty(); });
        if (stop && ready.empty() && running.empty()) return;
        while (!ready.empty() && !free_slots.empty()) {
          Request* r = ready.front();
          ready.pop_front();
          r->slot = free_slots.back();
          free_slots.pop_back();
          r->state = KH_REQ_RUNNING;
          running.push_back(r);
        }
      }
      // issue: keep two quanta in flight per request
      for (Request* r : running) {
        while (!stop && r->status == KH_OK && r->inflight < 2 && r->issued < r->nsteps) {
          if (!r->ev[0]) {
            cudaEventCreateWithFlags(&r->ev[0], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&r->ev[1], cudaEventDisableTiming);
          }
          // quanta are whole multiples of the request's step alignment, so its
          // batches repeat and replay captured step graphs
          const int64_t al = std::max(1, r->sim->impl->step_alignment());
          const int64_t quantum = std::max<int64_t>(al, (desc.quantum_steps + al - 1) / al * al);
          const int64_t q = std::min<int64_t>(quantum, r->nsteps - r->issued);
          if (r->t_start < 0) {
            std::lock_guard<std::mutex> g(mu);
            r->t_start = now();
          }
          const kh_status st = r->sim->impl->step(q, streams[r->slot]);
          if (st != KH_OK) {
            r->status = st;
            r->error = r->sim->impl->err;
            break;
          }
          cudaEventRecord(r->ev[(r->head + r->inflight) & 1], streams[r->slot]);
          ++r->inflight;
          r->issued += q;
        }
      }
      // retire finished quanta and requests
      bool progress = false;
      for (size_t i = 0; i < running.size();) {
        Request* r = running[i];
        while (r->inflight > 0 && cudaEventQuery(r->ev[r->head]) == cudaSuccess) {
          r->head ^= 1;
          --r->inflight;
          progress = true;
        }
        const bool ended = r->inflight == 0 && (r->issued >= r->nsteps || r->status != KH_OK || stop);
        if (!ended) {
          ++i;
          continue;
        }
        kh_status st = r->status;
        std::string msg = r->error;
        if (st == KH_OK) {
          st = r->sim->impl->wait_idle();  // all quanta done: reads the device error flag
          if (st != KH_OK) msg = r->sim->impl->err;
          else if (r->issued < r->nsteps) {
            st = KH_ERR_INVALID;
            msg = "server stopped before the request finished";
          }
        }
        for (auto& e : r->ev)
          if (e) {
            cudaEventDestroy(e);
            e = nullptr;
          }
        {
          std::lock_guard<std::mutex> g(mu);
          free_slots.push_back(r->slot);
          r->slot = -1;
          finish(r, st, msg);
        }
        running[i] = running.back();
        running.pop_back();
        progress = true;
      }
      if (!progress && !running.empty()) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
  }
};

extern "C" {

kh_status kh_server_create(const kh_server_desc* d, kh_server** out) {
  if (!d || !out) return KH_ERR_INVALID;
  *out = nullptr;
  if (d->budget_bytes <= 0 || d->max_resident < 0 || d->quantum_steps < 0) return KH_ERR_INVALID;
  std::unique_ptr<kh_server> s(new (std::nothrow) kh_server());
  if (!s) return KH_ERR_OOM;
  s->desc = *d;
  if (s->desc.max_resident == 0) s->desc.max_resident = 16;
  if (s->desc.quantum_steps == 0) s->desc.quantum_steps = 64;
  if (cudaGetDevice(&s->device) != cudaSuccess) return KH_ERR_CUDA;
  s->t0 = Clock::now();
  for (int i = 0; i < s->desc.max_resident; ++i) {
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
      return KH_ERR_CUDA;
    }
    s->streams.push_back(st);
    s->free_slots.push_back(s->desc.max_resident - 1 - i);
  }
  kh_server* raw = s.release();
  raw->admit_thr = std::thread([raw] { raw->admit_loop(); });
  raw->step_thr = std::thread([raw] { raw->step_loop(); });
  *out = raw;
  return KH_OK;
}

kh_status kh_server_submit(kh_server* s, kh_sim* sim, int64_t nsteps, int64_t* ticket) {
  if (!s || !sim || !ticket || nsteps < 0) return KH_ERR_INVALID;
  if (sim->impl->is_prepared()) {
    std::lock_guard<std::mutex> g(s->mu);
    s->err = "submit takes a simulation that has not been prepared";
    return KH_ERR_INVALID;
  }
  const int64_t est = sim->impl->estimate_bytes();
  std::lock_guard<std::mutex> g(s->mu);
  if (s->stop) return KH_ERR_INVALID;
  if (est > s->desc.budget_bytes) {
    s->err = "request needs " + std::to_string(est) + " bytes, more than the whole budget";
    return KH_ERR_OOM;
  }
  auto r = std::make_unique<Request>();
  r->ticket = s->next_ticket++;
  r->sim = sim;
  r->nsteps = nsteps;
  r->est_bytes = est;
  r->t_submit = s->now();
  *ticket = r->ticket;
  s->pending.push_back(r.get());
  s->reqs[r->ticket] = std::move(r);
  s->cv_admit.notify_all();
  return KH_OK;
}

kh_status kh_server_wait(kh_server* s, int64_t ticket, double timeout_s) {
  if (!s) return KH_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return KH_ERR_INVALID;
  Request* r = it->second.get();
  auto done = [&] { return r->state == KH_REQ_DONE || r->state == KH_REQ_FAILED; };
  if (timeout_s < 0) s->cv_done.wait(lk, done);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) return KH_ERR_TIMEOUT;
  return r->status;
}

kh_status kh_server_wait_any(kh_server* s, double timeout_s, int64_t* ticket) {
  if (!s || !ticket) return KH_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto any = [&] { return !s->done_q.empty(); };
  if (timeout_s < 0) s->cv_done.wait(lk, any);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), any)) return KH_ERR_TIMEOUT;
  *ticket = s->done_q.front();
  s->done_q.pop_front();
  return KH_OK;
}

kh_status kh_server_info(kh_server* s, int64_t ticket, kh_request_info* out) {
  if (!s || !out) return KH_ERR_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return KH_ERR_INVALID;
  const Request* r = it->second.get();
  out->state = r->state;
  out->status = r->status;
  out->steps = r->nsteps;
  out->bytes = r->est_bytes;
  out->t_submit = r->t_submit;
  out->t_admit = r->t_admit;
  out->t_start = r->t_start;
  out->t_done = r->t_done;
  return KH_OK;
}

kh_status kh_server_release(kh_server* s, int64_t ticket) {
  if (!s) return KH_ERR_INVALID;
  kh_sim* sim = nullptr;
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return KH_ERR_INVALID;
    Request* r = it->second.get();
    if (r->state != KH_REQ_DONE && r->state != KH_REQ_FAILED) {
      s->err = "release of a request that has not finished";
      return KH_ERR_INVALID;
    }
    sim = r->sim;
    r->sim = nullptr;
    r->state = KH_REQ_RELEASED;
  }
  const int64_t bytes = sim->impl->device_bytes();
  kh_sim_destroy(sim);
  std::lock_guard<std::mutex> g(s->mu);
  s->budget_used -= bytes;
  s->reqs.erase(ticket);
  s->cv_admit.notify_all();
  return KH_OK;
}

kh_status kh_server_stats(kh_server* s, int64_t* queued, int64_t* resident, int64_t* budget_used) {
  if (!s) return KH_ERR_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  if (queued) *queued = int64_t(s->pending.size());
  if (resident) *resident = s->resident;
  if (budget_used) *budget_used = s->budget_used;
  return KH_OK;
}

const char* kh_server_last_error(const kh_server* s) { return s ? s->err.c_str() : "null server"; }

void kh_server_destroy(kh_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_admit.notify_all();
  s->cv_step.notify_all();
  if (s->admit_thr.joinable()) s->admit_thr.join();
  if (s->step_thr.joinable()) s->step_thr.join();
  for (auto& kv : s->reqs)
    if (kv.second->sim) kh_sim_destroy(kv.second->sim);
  for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
  delete s;
}

}  // extern "C"
