// gd_server.cpp -- request server with continuous batching (host code).
//
// No counterpart in the reference, which clusters one data set per program
// run.  Requests (one clustering instance each, host buffers) are queued;
// `workers` threads each own a gbdbscan context and CUDA stream.  A worker that
// is free takes every queued request it may admit -- first in, first out,
// while the estimated device memory of all requests in flight stays within
// the HBM budget and the batch stays within max_batch -- and clusters them
// together with gd_batch_dbscan.  Requests that arrive while the workers are
// busy wait for the next free worker, so the GPU always holds the work of up
// to `workers` batches, overlapping on their streams.  Every request's labels
// equal gd_dbscan's on that request alone (the batch path computes each
// instance independently).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gbdbscan.h"

namespace gdio {
void set_error(const std::string& m);
}

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point t0, Clock::time_point t) {
  return std::chrono::duration<double, std::milli>(t - t0).count();
}

// device bytes one point of a request may need during a run (buffers of the
// build and expand stages, cell tables and row hash, generously rounded)
constexpr int64_t kBytesPerPoint = 320;
constexpr int64_t kBytesPerRequest = 1 << 16;

struct Request {
  int64_t id = 0;
  gd_instance inst{};
  const double* coords = nullptr;
  int32_t* labels = nullptr;
  int64_t bytes = 0;
  int state = 0;  // 0 queued, 1 running, 2 done
  gd_status status = GD_OK;
  int64_t clusters = 0;
  int32_t batch_size = 0;
  std::string msg;  // failure message of the batch that ran this request
  Clock::time_point t_submit, t_start, t_done;
};

}  // namespace

struct gd_server {
  gd_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_work;  // workers wait for requests
  std::condition_variable cv_done;  // waiters wait for completions
  std::deque<int64_t> queue;
  std::unordered_map<int64_t, Request> reqs;
  int64_t next_id = 1;
  int64_t inflight_bytes = 0;
  bool stop = false;
  int starting = 0;  // workers still creating their context
  int alive = 0;     // workers with a context
  std::vector<std::thread> threads;
  Clock::time_point t0 = Clock::now();
  gd_server_stats stats{};
  std::string error;

  void worker(int w);
};

void gd_server::worker(int w) {
  gd_ctx* ctx = nullptr;
  const bool ok = cudaSetDevice(cfg.device) == cudaSuccess &&
                  gd_ctx_create(cfg.device, &ctx) == GD_OK &&
                  gd_ctx_set_precision(ctx, cfg.precision) == GD_OK;
  {
    std::lock_guard<std::mutex> lock(mu);
    starting -= 1;
    if (ok) alive += 1;
    else error = std::string("server worker ") + std::to_string(w) + ": " + gd_last_error();
  }
  cv_done.notify_all();
  if (!ok) {
    if (ctx) gd_ctx_destroy(ctx);
    return;
  }
  std::vector<gd_instance> inst;
  std::vector<int64_t> counts;
  std::vector<Request*> rp;
  double* stage_in = nullptr;
  int32_t* stage_out = nullptr;
  size_t cap_in = 0, cap_out = 0;
  // grows a pinned staging buffer; false when the host allocation fails
  auto reserve = [](auto*& buf, size_t& cap, size_t want) {
    if (want <= cap) return true;
    if (buf) cudaFreeHost(buf);
    cap = std::max(want, cap * 2);
    if (cudaHostAlloc((void**)&buf, cap * sizeof(*buf), cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      buf = nullptr;
      cap = 0;
      return false;
    }
    return true;
  };
  // clusters rp[b, e) as one batch; fills status, clusters and labels
  auto run = [&](size_t b, size_t e) {
    size_t nd = 0, np = 0;
    inst.clear();
    for (size_t j = b; j < e; ++j) {
      inst.push_back(rp[j]->inst);
      nd += (size_t)rp[j]->inst.n * rp[j]->inst.dim;
      np += (size_t)rp[j]->inst.n;
    }
    gd_status st = GD_OK;
    std::string msg;
    if (!reserve(stage_in, cap_in, nd) || !reserve(stage_out, cap_out, np)) {
      st = GD_ENOMEM;
      msg = "server: pinned host staging allocation failed";
    }
    if (st == GD_OK) {
      size_t off = 0;
      for (size_t j = b; j < e; ++j) {
        const size_t cnt = (size_t)rp[j]->inst.n * rp[j]->inst.dim;
        if (cnt) memcpy(stage_in + off, rp[j]->coords, cnt * 8);
        off += cnt;
      }
      counts.assign(e - b, 0);
      st = gd_batch_dbscan(ctx, (int32_t)(e - b), inst.data(), stage_in, 0, stage_out,
                           counts.data(), nullptr);
      if (st != GD_OK) msg = gd_last_error();
    }
    size_t off = 0;
    for (size_t j = b; j < e; ++j) {
      Request* r = rp[j];
      r->status = st;
      r->msg = msg;
      r->clusters = st == GD_OK ? counts[j - b] : 0;
      r->batch_size = (int32_t)(e - b);
      if (st == GD_OK && r->inst.n) memcpy(r->labels, stage_out + off, (size_t)r->inst.n * 4);
      off += (size_t)r->inst.n;
    }
    return st;
  };
  while (true) {
    int64_t batch_bytes = 0;
    rp.clear();
    {
      std::unique_lock<std::mutex> lock(mu);
      cv_work.wait(lock, [&] { return stop || !queue.empty(); });
      if (stop && queue.empty()) break;
      // admit first in, first out while the budget allows; a request larger
      // than the whole budget runs alone once nothing else is in flight
      while (!queue.empty() && (int)rp.size() < cfg.max_batch) {
        Request& r = reqs[queue.front()];
        const bool fits = inflight_bytes + batch_bytes + r.bytes <= cfg.hbm_budget_bytes;
        const bool alone = inflight_bytes == 0 && rp.empty();
        if (!fits && !alone) break;
        batch_bytes += r.bytes;
        r.state = 1;
        r.t_start = Clock::now();
        rp.push_back(&r);
        queue.pop_front();
      }
      if (rp.empty()) {
        // nothing admissible yet: wait for a completion to free budget
        cv_done.wait_for(lock, std::chrono::milliseconds(1));
        continue;
      }
      inflight_bytes += batch_bytes;
    }
    // a failed batch (device memory, say) is retried one request at a time,
    // so one request cannot fail the others
    if (run(0, rp.size()) != GD_OK && rp.size() > 1)
      for (size_t j = 0; j < rp.size(); ++j) run(j, j + 1);
    {
      std::lock_guard<std::mutex> lock(mu);
      const auto now = Clock::now();
      int64_t np = 0, bad = 0;
      for (Request* r : rp) {
        r->state = 2;
        r->t_done = now;
        np += r->inst.n;
        if (r->status != GD_OK) {
          bad += 1;
          error = r->msg;
        }
      }
      inflight_bytes -= batch_bytes;
      stats.batches += 1;
      stats.completed += (int64_t)rp.size();
      stats.failed += bad;
      stats.points += np;
      stats.max_batch_seen = std::max<int64_t>(stats.max_batch_seen, (int64_t)rp.size());
    }
    cv_done.notify_all();
    cv_work.notify_all();
  }
  if (stage_in) cudaFreeHost(stage_in);
  if (stage_out) cudaFreeHost(stage_out);
  gd_ctx_destroy(ctx);
  std::lock_guard<std::mutex> lock(mu);
  alive -= 1;
}

extern "C" {

gd_status gd_server_create(const gd_server_config* cfg, gd_server** out) {
  if (!cfg || !out) {
    gdio::set_error("gd_server_create: NULL argument");
    return GD_EINVAL;
  }
  *out = nullptr;
  if (cfg->workers < 1 || cfg->workers > 16 || cfg->max_batch < 1 || cfg->hbm_budget_bytes <= 0 ||
      (cfg->precision != GD_PREC_FP64 && cfg->precision != GD_PREC_FP32_BAND)) {
    gdio::set_error("gd_server_create: workers must be 1..16, max_batch >= 1, budget > 0, "
                    "precision a gd_precision");
    return GD_EINVAL;
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || cfg->device < 0 || cfg->device >= count) {
    cudaGetLastError();
    gdio::set_error("gd_server_create: no such CUDA device");
    return GD_ENODEV;
  }
  gd_server* s = new gd_server();
  s->cfg = *cfg;
  s->starting = cfg->workers;
  for (int w = 0; w < cfg->workers; ++w) s->threads.emplace_back(&gd_server::worker, s, w);
  bool any;
  std::string err;
  {
    std::unique_lock<std::mutex> lock(s->mu);
    s->cv_done.wait(lock, [&] { return s->starting == 0; });
    any = s->alive > 0;
    err = s->error;
  }
  if (!any) {
    gd_server_destroy(s);
    gdio::set_error("gd_server_create: " + err);
    return GD_ECUDA;
  }
  *out = s;
  return GD_OK;
}

void gd_server_destroy(gd_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->threads) t.join();
  delete s;
}

gd_status gd_server_submit(gd_server* s, const gd_instance* inst, const double* coords,
                           int32_t* labels, int64_t* request_id) {
  if (!s || !inst || !request_id || (inst->n > 0 && (!coords || !labels))) {
    gdio::set_error("gd_server_submit: NULL argument");
    return GD_EINVAL;
  }
  if (inst->n < 0 || (inst->dim != 2 && inst->dim != 3) || !(inst->eps > 0) ||
      inst->minpts < 1) {
    gdio::set_error("gd_server_submit: bad instance (n, dim, eps or minpts)");
    return GD_EINVAL;
  }
  // reject bad coordinates here, so that they cannot fail a whole batch
  for (int64_t i = 0; i < inst->n * inst->dim; ++i)
    if (!std::isfinite(coords[i])) {
      gdio::set_error("gd_server_submit: coordinate " + std::to_string(i) + " is not finite");
      return GD_EINVAL;
    }
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->alive == 0) {
    gdio::set_error("gd_server_submit: no worker is running");
    return GD_ESTATE;
  }
  Request r;
  r.id = s->next_id++;
  r.inst = *inst;
  r.coords = coords;
  r.labels = labels;
  r.bytes = kBytesPerRequest + inst->n * kBytesPerPoint;
  r.t_submit = Clock::now();
  s->reqs[r.id] = r;
  s->queue.push_back(r.id);
  s->stats.submitted += 1;
  *request_id = r.id;
  s->cv_work.notify_one();
  return GD_OK;
}

gd_status gd_server_wait(gd_server* s, int64_t id, double timeout_ms, gd_request_info* info) {
  if (!s) {
    gdio::set_error("gd_server_wait: NULL server");
    return GD_EINVAL;
  }
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) {
    gdio::set_error("gd_server_wait: unknown request id");
    return GD_EINVAL;
  }
  auto done = [&] { return s->reqs[id].state == 2; };
  if (timeout_ms < 0) s->cv_done.wait(lock, done);
  else if (!s->cv_done.wait_for(lock, std::chrono::duration<double, std::milli>(timeout_ms), done)) {
    gdio::set_error("gd_server_wait: request not finished within the timeout");
    return GD_ETIMEOUT;
  }
  Request& r = s->reqs[id];
  if (info) {
    info->n_clusters = r.clusters;
    info->status = r.status;
    info->batch_size = r.batch_size;
    info->submit_ms = ms_since(s->t0, r.t_submit);
    info->start_ms = ms_since(s->t0, r.t_start);
    info->done_ms = ms_since(s->t0, r.t_done);
  }
  const gd_status st = r.status;
  if (st != GD_OK) gdio::set_error(r.msg);
  s->reqs.erase(id);
  return st;
}

gd_status gd_server_get_stats(gd_server* s, gd_server_stats* out) {
  if (!s || !out) {
    gdio::set_error("gd_server_get_stats: NULL argument");
    return GD_EINVAL;
  }
  std::lock_guard<std::mutex> lock(s->mu);
  *out = s->stats;
  out->queued = (int64_t)s->queue.size();
  out->inflight_bytes = s->inflight_bytes;
  return GD_OK;
}

}  // extern "C"
