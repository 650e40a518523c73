// pn_server.cu -- served solves: continuous batching of requests into waves on one GPU.
//
// A request is a list of solves (one reconstruction iteration's beam positions x energies, the
// inner loop of scripts/2d_full_reconstruction_test.jl:104-149).  One scheduler thread per server:
//
//   * requests wait in arrival order; whenever a wave slot is free and the memory budget has room,
//     the scheduler takes the waiting requests from the head (same precision and mode, up to a
//     solve limit) and makes them one wave: a pn_batch whose device memory -- tables, tapes,
//     checkpoints, inputs and outputs -- is carved from the server's arena;
//   * each wave runs on its own stream (its groups on streams forked from it), so waves admitted
//     while others are still on the GPU overlap with them;
//   * a host function queued behind the wave tells the scheduler when it is done; the scheduler
//     copies the outputs to the caller's buffers, returns the wave's ranges to the arena and wakes
//     the waiters, and the freed room admits the next waiting requests.
//
// No wave ever synchronises the device: the arena has no cudaFree, uploads go on the wave's
// streams, and the scheduler waits only on the stream of a wave that is already complete.  A
// wave that does not fit goes back to the queue until running waves release memory; a single
// request that does not fit an otherwise idle server fails with PN_ERR_NO_MEMORY.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/pnepma.h"
#include "pn_arena.h"
#include "pn_batch_impl.h"

namespace pn {
void set_last_error(const std::string& msg);
}

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
  uint64_t id = 0;
  int n = 0;
  int adjoint = 0;
  int precision = 0;
  std::vector<std::pair<int, int>> key;   // sorted distinct (order, active axes) of its solves
  std::vector<const pn_desc*> descs;
  std::vector<const double*> rho, noa, acs, ibar;
  std::vector<double*> I, rho_bar, noa_bar, acs_bar;
  bool done = false;
  int status = PN_OK;
  int wave = -1;
  std::string err;
  Clock::time_point t_submit, t_admit, t_done;
};

struct Wave {
  int id = 0;
  pn_batch* b = nullptr;
  cudaStream_t st = nullptr;
  std::vector<Request*> reqs;
  std::vector<void*> ranges;   // arena ranges of the inputs and outputs
  std::vector<pn_sizes> sizes; // per solve, in wave order
  std::vector<const double*> rho, noa, acs, ibar;
  std::vector<double*> I, rho_bar, noa_bar, acs_bar;
  int adjoint = 0;
  int rc = PN_OK;
  std::string err;
};

}  // namespace

struct pn_server {
  int device = 0;
  char* base = nullptr;
  std::unique_ptr<pn::Arena> arena;
  int max_waves = 8;
  int max_wave_solves = 1024;
  int K = 0;

  std::mutex mu;
  std::condition_variable cv;        // scheduler wake-up: submissions, finished waves, stop
  std::condition_variable done_cv;   // waiters in pn_wait
  bool stop = false;
  bool mem_blocked = false;          // the head of the queue waits for memory
  std::deque<Request*> pending;
  std::vector<Wave*> finished;       // waves whose host function ran
  std::unordered_map<uint64_t, std::unique_ptr<Request>> requests;
  uint64_t next_id = 1;
  int next_wave = 0;
  int in_flight = 0;
  int max_in_flight = 0;
  long long submitted = 0, completed = 0, solves_done = 0, waves = 0;
  double build_us = 0.0;
  std::thread worker;

  void run();
  int launch_wave(Wave* w);
  void finish_wave(Wave* w);
};

namespace {

void CUDART_CB wave_done(void* p) {
  // runs on a CUDA driver thread: no CUDA calls here
  auto* pair = static_cast<std::pair<pn_server*, Wave*>*>(p);
  pn_server* s = pair->first;
  Wave* w = pair->second;
  delete pair;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->finished.push_back(w);
  }
  s->cv.notify_all();
}

template <class P>
int upload_dedup(pn::Arena* arena, Wave* w, std::map<std::pair<const void*, long long>, P>& seen, const double* host,
                 long long cnt, P& out, std::string& err) {
  auto key = std::make_pair((const void*)host, cnt);
  auto it = seen.find(key);
  if (it != seen.end()) {
    out = it->second;
    return PN_OK;
  }
  void* d = arena->alloc((size_t)std::max<long long>(cnt, 1) * sizeof(double));
  if (!d) {
    err = "no room in the memory budget for the inputs";
    return PN_ERR_NO_MEMORY;
  }
  w->ranges.push_back(d);
  if (cnt > 0 && cudaMemcpyAsync(d, host, sizeof(double) * (size_t)cnt, cudaMemcpyHostToDevice, w->st) != cudaSuccess) {
    cudaGetLastError();
    err = "input upload failed";
    return PN_ERR_CUDA;
  }
  out = (P)d;
  seen[key] = out;
  return PN_OK;
}

int alloc_out(pn::Arena* arena, Wave* w, long long cnt, double*& out, std::string& err) {
  void* d = arena->alloc((size_t)std::max<long long>(cnt, 1) * sizeof(double));
  if (!d) {
    err = "no room in the memory budget for the outputs";
    return PN_ERR_NO_MEMORY;
  }
  w->ranges.push_back(d);
  out = (double*)d;
  return PN_OK;
}

}  // namespace

// Build the wave's batch in the arena, upload its inputs and queue its work; called without the
// lock.  On failure everything the wave holds is released and the code returned.
int pn_server::launch_wave(Wave* w) {
  const bool trace = std::getenv("PN_TRACE") != nullptr;
  const auto t_begin = Clock::now();
  std::vector<const pn_desc*> descs;
  for (Request* r : w->reqs) descs.insert(descs.end(), r->descs.begin(), r->descs.end());
  const int n = (int)descs.size();
  auto release = [&]() {
    // uploads into the wave's ranges may still be in flight
    if (w->st) cudaStreamSynchronize(w->st);
    if (w->b) pn_batch_destroy(w->b);
    w->b = nullptr;
    for (void* p : w->ranges) arena->free(p);
    w->ranges.clear();
    if (w->st) cudaStreamDestroy(w->st);
    w->st = nullptr;
  };
  if (cudaStreamCreateWithFlags(&w->st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    w->err = "stream creation failed";
    return PN_ERR_CUDA;
  }
  // inputs and outputs first, so the tapes get what is left
  w->sizes.resize(n);
  w->rho.resize(n); w->noa.resize(n); w->acs.resize(n); w->ibar.resize(n);
  w->I.resize(n); w->rho_bar.resize(n); w->noa_bar.resize(n); w->acs_bar.resize(n);
  std::map<std::pair<const void*, long long>, const double*> seen;
  int q = 0;
  for (Request* r : w->reqs)
    for (int i = 0; i < r->n; ++i, ++q) {
      int rc = pn_query_sizes(r->descs[i], &w->sizes[q]);
      if (rc) {
        w->err = pn_last_error(nullptr);
        release();
        return rc;
      }
      const pn_sizes& z = w->sizes[q];
      const long long nr = r->descs[i]->n_xrays;
      if ((rc = upload_dedup(arena.get(), w, seen, r->rho[i], z.n_rho, w->rho[q], w->err)) ||
          (rc = upload_dedup(arena.get(), w, seen, r->noa[i], z.n_noa, w->noa[q], w->err)) ||
          (rc = upload_dedup(arena.get(), w, seen, r->acs[i], z.n_acs, w->acs[q], w->err)) ||
          (rc = alloc_out(arena.get(), w, nr, w->I[q], w->err))) {
        release();
        return rc;
      }
      if (w->adjoint) {
        if ((rc = upload_dedup(arena.get(), w, seen, r->ibar[i], nr, w->ibar[q], w->err)) ||
            (rc = alloc_out(arena.get(), w, z.n_rho, w->rho_bar[q], w->err)) ||
            (rc = alloc_out(arena.get(), w, z.n_noa, w->noa_bar[q], w->err)) ||
            (rc = alloc_out(arena.get(), w, z.n_acs, w->acs_bar[q], w->err))) {
          release();
          return rc;
        }
      }
    }
  const auto t_io = Clock::now();
  // tapes: a fair share of what is free among the wave slots still open or, for a wave whose every
  // state would not fit that share, up to half of what is free (its adjoint then recomputes fewer
  // forward steps; a batch takes only what its tape needs).  "Does not fit" from the stride search
  // wants a larger budget, a full arena (tables and tiles come on top of the tapes) a smaller one,
  // i.e. a longer checkpoint stride.
  const long long free_now = (long long)arena->free_bytes();
  const int open = std::max(1, max_waves - in_flight);
  long long need = 0;   // every state of every solve (the device layout's padding estimated)
  for (int q = 0; q < n; ++q)
    need += (long long)(descs[q]->n_steps + 1) * w->sizes[q].n_state * (descs[q]->precision == PN_FP32 ? 4 : 8);
  need += need / 16;
  const long long fair = free_now / open;
  std::vector<long long> tries = {std::max(fair, std::min(need, free_now / 2))};
  for (long long b : {fair, free_now * 3 / 4, free_now / 2, free_now / 4, free_now / 8})
    if (std::find(tries.begin(), tries.end(), b) == tries.end()) tries.push_back(b);
  int rc = PN_ERR_NO_MEMORY;
  for (long long budget : tries) {
    std::string err;
    const auto t_try = Clock::now();
    rc = pn::batch_create(descs.data(), n, budget, K, 0, arena.get(), &w->b, err);
    if (trace)
      std::fprintf(stderr, "[pn] wave %d: %d solves, budget %.1f GB: %s (%.1f ms)\n", w->id, n, budget / 1e9,
                   rc == PN_OK ? "built" : err.c_str(), ms_between(t_try, Clock::now()));
    if (rc == PN_OK) break;
    w->err = err;
    if (rc != PN_ERR_NO_MEMORY) break;
  }
  if (rc) {
    release();
    return rc;
  }
  const auto t_built = Clock::now();
  rc = pn_batch_forward(w->b, w->rho.data(), w->noa.data(), w->acs.data(), w->I.data(), w->st);
  const auto t_fwd = Clock::now();
  if (rc == PN_OK && w->adjoint)
    rc = pn_batch_adjoint(w->b, w->ibar.data(), w->rho_bar.data(), w->noa_bar.data(), w->acs_bar.data(), w->st);
  if (trace)
    std::fprintf(stderr, "[pn] wave %d: forward launched in %.1f ms, adjoint in %.1f ms\n", w->id,
                 ms_between(t_built, t_fwd), ms_between(t_fwd, Clock::now()));
  if (rc) {
    w->err = pn_last_error(nullptr);
    // a group that failed part-way is not joined to the wave's stream: wait for all its work
    cudaDeviceSynchronize();
    release();
    return rc;
  }
  if (trace)
    std::fprintf(stderr, "[pn] wave %d: inputs %.1f ms, build+launch %.1f ms, arena %.1f / %.1f GB\n", w->id,
                 ms_between(t_begin, t_io), ms_between(t_io, Clock::now()), arena->used() / 1e9, arena->size() / 1e9);
  auto* arg = new std::pair<pn_server*, Wave*>(this, w);
  if (cudaLaunchHostFunc(w->st, wave_done, arg) != cudaSuccess) {
    delete arg;
    cudaGetLastError();
    w->err = "cudaLaunchHostFunc failed";
    release();
    return PN_ERR_CUDA;
  }
  return PN_OK;
}

// Copy a complete wave's outputs to the callers and release it; called without the lock.
void pn_server::finish_wave(Wave* w) {
  int rc = PN_OK;
  std::string err;
  int q = 0;
  for (Request* r : w->reqs)
    for (int i = 0; i < r->n && rc == PN_OK; ++i, ++q) {
      const pn_sizes& z = w->sizes[q];
      const long long nr = r->descs[i]->n_xrays;
      cudaError_t e = cudaMemcpyAsync(r->I[i], w->I[q], sizeof(double) * nr, cudaMemcpyDeviceToHost, w->st);
      if (w->adjoint && e == cudaSuccess) {
        e = cudaMemcpyAsync(r->rho_bar[i], w->rho_bar[q], sizeof(double) * z.n_rho, cudaMemcpyDeviceToHost, w->st);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(r->noa_bar[i], w->noa_bar[q], sizeof(double) * z.n_noa, cudaMemcpyDeviceToHost, w->st);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(r->acs_bar[i], w->acs_bar[q], sizeof(double) * z.n_acs, cudaMemcpyDeviceToHost, w->st);
      }
      if (e != cudaSuccess) {
        rc = PN_ERR_CUDA;
        err = std::string("output copy failed: ") + cudaGetErrorString(e);
      }
    }
  cudaError_t e = cudaStreamSynchronize(w->st);
  if (e != cudaSuccess && rc == PN_OK) {
    rc = PN_ERR_CUDA;
    err = std::string("wave failed on the device: ") + cudaGetErrorString(e);
  }
  if (rc == PN_OK) {
    const int st = pn::batch_status(w->b);
    if (st != PN_OK) {
      rc = st;
      err = "a bounded device-side wait of the wave ran out";
    }
  }
  pn_batch_destroy(w->b);
  w->b = nullptr;
  for (void* p : w->ranges) arena->free(p);
  w->ranges.clear();
  cudaStreamDestroy(w->st);
  w->st = nullptr;
  w->rc = rc;
  w->err = err;
}

void pn_server::run() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    cv.wait(lk, [&] {
      return !finished.empty() || (stop && in_flight == 0) ||
             (!stop && !pending.empty() && !mem_blocked && in_flight < max_waves);
    });
    // completions first: they free slots and memory
    while (!finished.empty()) {
      Wave* w = finished.back();
      finished.pop_back();
      lk.unlock();
      finish_wave(w);
      const auto t = Clock::now();
      lk.lock();
      for (Request* r : w->reqs) {
        r->status = w->rc;
        r->err = w->err;
        r->t_done = t;
        r->done = true;
        ++completed;
        solves_done += r->n;
      }
      --in_flight;
      mem_blocked = false;
      delete w;
      done_cv.notify_all();
    }
    if (stop) {
      // requests never admitted fail; in-flight waves are waited for
      for (Request* r : pending) {
        r->status = PN_ERR_STATE;
        r->err = "the server was destroyed before the request ran";
        r->t_done = Clock::now();
        r->done = true;
      }
      pending.clear();
      done_cv.notify_all();
      if (in_flight == 0) return;
      continue;
    }
    // admissions
    int limit = max_wave_solves;
    while (!pending.empty() && !mem_blocked && in_flight < max_waves) {
      Wave* w = new Wave;
      w->id = next_wave++;
      // the head and every later waiting request of the same kind (precision, mode, and set of
      // (order, active axes)): a wave completes as a whole, so kinds of very different cost are
      // not mixed, and a kind's later arrivals join the head's wave instead of waiting for a slot
      Request* head = pending.front();
      w->adjoint = head->adjoint;
      int solves = 0;
      for (auto it = pending.begin(); it != pending.end();) {
        Request* r = *it;
        if (r->precision != head->precision || r->adjoint != head->adjoint || r->key != head->key) {
          ++it;
          continue;
        }
        if (!w->reqs.empty() && solves + r->n > limit) break;
        w->reqs.push_back(r);
        solves += r->n;
        it = pending.erase(it);
      }
      ++in_flight;
      lk.unlock();
      const auto t = Clock::now();
      int rc = launch_wave(w);
      const auto tb = Clock::now();
      lk.lock();
      build_us += 1e3 * ms_between(t, tb);
      if (rc == PN_OK) {
        for (Request* r : w->reqs) {
          r->t_admit = t;
          r->wave = w->id;
        }
        ++waves;
        max_in_flight = std::max(max_in_flight, in_flight);
        limit = max_wave_solves;
        continue;
      }
      --in_flight;
      if (rc == PN_ERR_NO_MEMORY && (w->reqs.size() > 1 || in_flight > 0)) {
        // back into the queue in arrival order: fewer requests per wave, or wait for running waves
        for (Request* r : w->reqs)
          pending.insert(std::upper_bound(pending.begin(), pending.end(), r,
                                          [](const Request* a, const Request* b) { return a->id < b->id; }),
                         r);
        if (w->reqs.size() > 1) limit = std::max(1, solves / 2);
        else mem_blocked = true;
        delete w;
        continue;
      }
      const auto td = Clock::now();
      for (Request* r : w->reqs) {
        r->status = rc;
        r->err = w->err;
        r->t_admit = t;
        r->t_done = td;
        r->done = true;
        ++completed;
      }
      delete w;
      done_cv.notify_all();
    }
  }
}

extern "C" {

int pn_server_create(const pn_server_options* options, pn_server** out) {
  if (!out) {
    pn::set_last_error("out is NULL");
    return PN_ERR_INVALID;
  }
  *out = nullptr;
  pn_server* s = nullptr;
  try {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
      cudaGetLastError();
      pn::set_last_error("no CUDA device is available");
      return PN_ERR_NO_DEVICE;
    }
    s = new pn_server;
    cudaGetDevice(&s->device);
    long long budget = options ? options->memory_budget : 0;
    if (options) {
      if (options->max_waves > 0) s->max_waves = options->max_waves;
      if (options->max_wave_solves > 0) s->max_wave_solves = options->max_wave_solves;
      if (options->checkpoint_stride < 0) {
        delete s;
        pn::set_last_error("checkpoint_stride must be >= 0");
        return PN_ERR_INVALID;
      }
      s->K = options->checkpoint_stride;
    }
    if (budget <= 0) {
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        delete s;
        pn::set_last_error("cudaMemGetInfo failed");
        return PN_ERR_CUDA;
      }
      budget = (long long)(fr / 2);
    }
    void* base = nullptr;
    if (cudaMalloc(&base, (size_t)budget) != cudaSuccess) {
      cudaGetLastError();
      delete s;
      pn::set_last_error("could not reserve the memory budget of " + std::to_string(budget) + " bytes");
      return PN_ERR_NO_MEMORY;
    }
    s->base = (char*)base;
    s->arena.reset(new pn::Arena(s->base, (size_t)budget));
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return PN_OK;
  } catch (const std::bad_alloc&) {
    if (s && s->base) cudaFree(s->base);
    delete s;
    pn::set_last_error("host allocation failed");
    return PN_ERR_NO_MEMORY;
  } catch (...) {
    if (s && s->base) cudaFree(s->base);
    delete s;
    pn::set_last_error("internal error");
    return PN_ERR_INVALID;
  }
}

int pn_submit(pn_server* s, const pn_request* req, uint64_t* ticket) {
  if (!s || !req || !ticket) {
    pn::set_last_error("NULL argument");
    return PN_ERR_INVALID;
  }
  try {
    const int n = req->n_solves;
    if (n < 1 || !req->descs || !req->rho || !req->noa || !req->acs || !req->intensities) {
      pn::set_last_error("a request needs n_solves >= 1, descriptors, inputs and intensities");
      return PN_ERR_INVALID;
    }
    if (req->adjoint && (!req->intensities_bar || !req->rho_bar || !req->noa_bar || !req->acs_bar)) {
      pn::set_last_error("an adjoint request needs intensities_bar, rho_bar, noa_bar and acs_bar");
      return PN_ERR_INVALID;
    }
    auto r = std::make_unique<Request>();
    r->n = n;
    r->adjoint = req->adjoint ? 1 : 0;
    for (int i = 0; i < n; ++i) {
      const pn_desc* d = req->descs[i];
      pn_sizes z;
      if (!d) {
        pn::set_last_error("descriptor is NULL");
        return PN_ERR_INVALID;
      }
      int rc = pn_query_sizes(d, &z);
      if (rc) return rc;   // message already set by pn_query_sizes
      if (i == 0) r->precision = d->precision;
      if (d->precision != r->precision) {
        pn::set_last_error("all solves of a request share one precision");
        return PN_ERR_INVALID;
      }
      if (!req->rho[i] || !req->noa[i] || !req->acs[i] || !req->intensities[i] ||
          (r->adjoint && (!req->intensities_bar[i] || !req->rho_bar[i] || !req->noa_bar[i] || !req->acs_bar[i]))) {
        pn::set_last_error("NULL buffer in the request");
        return PN_ERR_INVALID;
      }
      int dims = 0;
      for (int k = 0; k < 3; ++k) dims |= (d->n_points[k] > 1 ? 1 : 0) << k;
      r->key.emplace_back(d->order, dims);
      r->descs.push_back(d);
      r->rho.push_back(req->rho[i]);
      r->noa.push_back(req->noa[i]);
      r->acs.push_back(req->acs[i]);
      r->I.push_back(req->intensities[i]);
      r->ibar.push_back(r->adjoint ? req->intensities_bar[i] : nullptr);
      r->rho_bar.push_back(r->adjoint ? req->rho_bar[i] : nullptr);
      r->noa_bar.push_back(r->adjoint ? req->noa_bar[i] : nullptr);
      r->acs_bar.push_back(r->adjoint ? req->acs_bar[i] : nullptr);
    }
    std::sort(r->key.begin(), r->key.end());
    r->key.erase(std::unique(r->key.begin(), r->key.end()), r->key.end());
    r->t_submit = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->stop) {
        pn::set_last_error("the server is shutting down");
        return PN_ERR_STATE;
      }
      r->id = s->next_id++;
      *ticket = r->id;
      s->pending.push_back(r.get());
      s->requests[r->id] = std::move(r);
      ++s->submitted;
    }
    s->cv.notify_all();
    return PN_OK;
  } catch (const std::bad_alloc&) {
    pn::set_last_error("host allocation failed");
    return PN_ERR_NO_MEMORY;
  } catch (...) {
    pn::set_last_error("internal error");
    return PN_ERR_INVALID;
  }
}

int pn_poll(pn_server* s, uint64_t ticket, pn_ticket_info* info) {
  if (!s || !info) {
    pn::set_last_error("NULL argument");
    return PN_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->requests.find(ticket);
  if (it == s->requests.end()) {
    pn::set_last_error("unknown ticket");
    return PN_ERR_INVALID;
  }
  const Request* r = it->second.get();
  info->done = r->done ? 1 : 0;
  info->status = r->done ? r->status : PN_OK;
  info->wave = r->wave;
  info->reserved = 0;
  info->queued_ms = r->wave >= 0 || r->done ? ms_between(r->t_submit, r->t_admit) : -1.0;
  info->total_ms = r->done ? ms_between(r->t_submit, r->t_done) : -1.0;
  if (r->done && r->status != PN_OK) pn::set_last_error(r->err);
  return PN_OK;
}

int pn_wait(pn_server* s, uint64_t ticket, int64_t timeout_ms) {
  if (!s) {
    pn::set_last_error("NULL argument");
    return PN_ERR_INVALID;
  }
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->requests.find(ticket);
  if (it == s->requests.end()) {
    pn::set_last_error("unknown ticket");
    return PN_ERR_INVALID;
  }
  Request* r = it->second.get();
  if (timeout_ms < 0) s->done_cv.wait(lk, [&] { return r->done; });
  else if (!s->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; })) {
    pn::set_last_error("the request is not done yet");
    return PN_ERR_TIMEOUT;
  }
  if (r->status != PN_OK) pn::set_last_error(r->err);
  return r->status;
}

int pn_server_query(pn_server* s, pn_server_info* info) {
  if (!s || !info) {
    pn::set_last_error("NULL argument");
    return PN_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  info->memory_budget = (int64_t)s->arena->size();
  info->bytes_in_use = (int64_t)s->arena->used();
  info->peak_bytes = (int64_t)s->arena->peak();
  info->requests_submitted = s->submitted;
  info->requests_done = s->completed;
  info->solves_done = s->solves_done;
  info->waves_launched = s->waves;
  info->waves_in_flight = s->in_flight;
  info->max_waves_in_flight = s->max_in_flight;
  info->wave_build_us = (int64_t)s->build_us;
  return PN_OK;
}

void pn_server_destroy(pn_server* s) {
  if (!s) return;
  try {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    if (s->base) cudaFree(s->base);
    delete s;
  } catch (...) {
  }
}

}  // extern "C"
