// Serving: a request loop over several lanes.
//
// Each lane is an ordinary context (its own stream and grow-only buffers)
// driven by its own host thread, so a batch on one lane overlaps on the GPU
// with batches on the others.  Requests wait in one queue, oldest first.  A
// free lane takes the oldest request it may serve and every later request
// of the same kind it may serve that fits beside it (continuous batching:
// whatever arrived while the lanes were busy forms the next batch), up to a
// request count and an optional byte cap, so that small requests do not wait
// for a large one's batch.  Express lanes serve only small requests.
// Admission counts the device memory of every lane -- what its context holds
// (grow-only), or the estimate of its running batch if that is larger --
// against the budget, and a batch that needs its lane to grow also needs that
// much free device memory (cudaMemGetInfo); a request larger than the whole
// budget runs alone once nothing else is in flight.
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <algorithm>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "wlgpu.h"

namespace {

using Clock = std::chrono::steady_clock;

int ceil_log2(unsigned x) {  // ceilLog2 (dwt_cpu.cc:75-78)
  if (x == 0) return 0;
  int n = 0;
  unsigned v = x - 1;
  while (v) { n++; v >>= 1; }
  return n;
}

long long padded(int len, int steps) {  // dwt_padded_length (dwt_cpu.cc:212-219)
  const long long mod = 1ll << steps;
  return mod * ((len - 1) / mod + 1);
}

int dtype_bytes(int dt) {
  switch (dt) {
    case WL_U8: return 1;
    case WL_U16: return 2;
    default: return 4;
  }
}

// Device working bytes of one request: two float coefficient buffers, the
// token slots and per-chunk records, staging of the input or output, plus a
// fixed allowance for tables.
double estimate(const wl_request &r) {
  if (r.kind == WL_REQ_COMPRESS) {
    const wl_cubelet &c = r.cubelet;
    long long n = 1;
    for (int a = 0; a < 3; a++) {
      const int m = ceil_log2((unsigned)c.size[a]);
      const int s = (c.params.steps[a] < 0 || c.params.steps[a] > m) ? m : c.params.steps[a];
      n *= padded(c.size[a], s);
    }
    const double in = (double)c.size[0] * c.size[1] * c.size[2] * dtype_bytes(c.dtype);
    return 12.0 * n + in + (1 << 20);
  }
  const wl_result *x = r.compressed;
  const double n = (double)x->size[0] * x->size[1] * x->size[2];
  const double out = (double)x->original_size[0] * x->original_size[1] * x->original_size[2] *
                     dtype_bytes(r.out_dtype);
  return 12.0 * n + 4.0 * x->n_words + out + (1 << 20);
}

// Bytes a request moves on the host side: its input (compress) or output
// (decompress); the size classes of the byte cap and the express lanes.
double request_bytes(const wl_request &r) {
  if (r.kind == WL_REQ_COMPRESS)
    return (double)r.cubelet.size[0] * r.cubelet.size[1] * r.cubelet.size[2] *
           dtype_bytes(r.cubelet.dtype);
  const wl_result *x = r.compressed;
  return (double)x->original_size[0] * x->original_size[1] * x->original_size[2] *
         dtype_bytes(r.out_dtype);
}

struct Job {
  unsigned long long id = 0;
  wl_request req;
  double est = 0;
  double bytes = 0;
  Clock::time_point submitted, started, finished;
  bool done = false;
  wl_status st = WL_OK;
  wl_result res;
  int batchSize = 0, lane = -1;
};

}  // namespace

struct wl_server {
  int device = 0;
  wl_serve_config cfg;
  std::mutex mu;
  std::condition_variable cvWork, cvDone;
  std::deque<Job *> pending;
  std::unordered_map<unsigned long long, Job *> jobs;
  double inflight = 0;          // estimates of the running batches
  std::vector<double> held;     // device bytes each lane's context holds
  std::vector<double> running;  // estimate of each lane's running batch (0: idle)
  bool stop = false;
  unsigned long long nextId = 1;
  std::vector<wl_ctx *> ctxs;
  std::vector<std::thread> workers;
  std::string err;
};

namespace {

wl_status serve_fail(wl_server *s, wl_status st, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (s) {
    std::lock_guard<std::mutex> g(s->mu);
    s->err = buf;
  }
  return st;
}

// Device bytes committed by the lanes other than `lane`.
double committed_others(const wl_server *s, int lane) {
  double c = 0;
  for (size_t l = 0; l < s->held.size(); l++)
    if ((int)l != lane) c += std::max(s->held[l], s->running[l]);
  return c;
}

bool any_running(const wl_server *s) {
  for (double r : s->running)
    if (r > 0) return true;
  return false;
}

bool express(const wl_server *s, int lane) { return lane < s->cfg.express_lanes; }

bool may_take(const wl_server *s, int lane, const Job *j) {
  return !express(s, lane) || j->bytes <= (double)s->cfg.small_request_bytes;
}

// Free device memory, refreshed at most every few milliseconds (the call
// goes through the driver).
double free_device_bytes(wl_server *s) {
  static thread_local Clock::time_point last;
  static thread_local double cached = 0;
  const Clock::time_point now = Clock::now();
  if (cached == 0 || now - last > std::chrono::milliseconds(5)) {
    size_t f = 0, t = 0;
    if (cudaSetDevice(s->device) == cudaSuccess && cudaMemGetInfo(&f, &t) == cudaSuccess)
      cached = (double)f;
    else
      cudaGetLastError();
    last = now;
  }
  return cached;
}

// Would a batch of estimate `est` fit on `lane` now?  A first request may
// always run when nothing else is in flight (alone: it gets what it needs);
// requests joining a batch must fit the budget in any case.
bool fits(wl_server *s, int lane, double est, bool first = true) {
  const double grow = std::max(0.0, est - s->held[lane]);
  if (first && !any_running(s)) return true;
  if (committed_others(s, lane) + std::max(s->held[lane], est) > (double)s->cfg.memory_budget)
    return false;
  // the lane's workspace grows only into memory the device has free
  constexpr double kMargin = 256.0 * (1 << 20);
  return grow == 0 || grow + kMargin <= free_device_bytes(s);
}

// The oldest request `lane` may serve, or the end of the queue.
std::deque<Job *>::iterator first_for(wl_server *s, int lane) {
  for (auto it = s->pending.begin(); it != s->pending.end(); ++it)
    if (may_take(s, lane, *it)) return it;
  return s->pending.end();
}

bool can_start(wl_server *s, int lane) {
  auto it = first_for(s, lane);
  return it != s->pending.end() && fits(s, lane, (*it)->est);
}

void worker(wl_server *s, int lane) {
  wl_ctx *ctx = s->ctxs[lane];
  std::vector<Job *> batch;
  std::vector<wl_cubelet> items;
  std::vector<wl_result> outs;
  for (;;) {
    batch.clear();
    double est = 0;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cvWork.wait(lk, [&] { return (s->stop && s->pending.empty()) || can_start(s, lane); });
      if (s->stop && s->pending.empty()) return;
      if (!can_start(s, lane)) continue;
      const double cap = (double)s->cfg.max_batch_bytes;
      auto it = first_for(s, lane);
      const int kind = (*it)->req.kind;
      const int dev = (*it)->req.out_on_device;
      double bytes = 0;
      // the oldest request this lane may serve, then every later one of its
      // kind (decompress: outputs all on the host or all on the device) that
      // fits beside it
      while (it != s->pending.end() && (int)batch.size() < s->cfg.max_batch) {
        Job *j = *it;
        const bool same = j->req.kind == kind &&
                          (kind != WL_REQ_DECOMPRESS || j->req.out_on_device == dev);
        const bool ok = batch.empty() ||
                        (same && may_take(s, lane, j) && (cap <= 0 || bytes + j->bytes <= cap) &&
                         fits(s, lane, est + j->est, false));
        if (!ok) {
          ++it;
          continue;
        }
        batch.push_back(j);
        est += j->est;
        bytes += j->bytes;
        it = s->pending.erase(it);
      }
      s->inflight += est;
      s->running[lane] = est;
      const Clock::time_point now = Clock::now();
      for (Job *j : batch) {
        j->started = now;
        j->batchSize = (int)batch.size();
        j->lane = lane;
      }
      // more work may fit beside this batch
      if (!s->pending.empty()) s->cvWork.notify_all();
    }

    if (batch[0]->req.kind == WL_REQ_DECOMPRESS) {
      const int n = (int)batch.size();
      std::vector<wl_result> rs(n);
      std::vector<int> dts(n);
      std::vector<void *> outs(n);
      for (int i = 0; i < n; i++) {
        rs[i] = *batch[i]->req.compressed;
        dts[i] = batch[i]->req.out_dtype;
        outs[i] = batch[i]->req.out;
      }
      wl_status st = wl_decompress_batch(ctx, rs.data(), n, dts.data(), outs.data(),
                                         batch[0]->req.out_on_device);
      // a bad request fails its batch: retry the batch one by one so the
      // others still succeed and the bad one gets its own status
      if (st != WL_OK && n > 1)
        for (Job *j : batch)
          j->st = wl_decompress_cubelet(ctx, j->req.compressed, j->req.out_dtype, j->req.out,
                                        j->req.out_on_device);
      else
        for (Job *j : batch) j->st = st;
    } else {
      const int n = (int)batch.size();
      items.resize(n);
      outs.assign(n, wl_result());
      for (int i = 0; i < n; i++) items[i] = batch[i]->req.cubelet;
      const wl_status st = wl_compress_batch(ctx, items.data(), n, 0, outs.data());
      for (int i = 0; i < n; i++) {
        batch[i]->st = st;
        if (st == WL_OK) batch[i]->res = outs[i];
      }
    }

    {
      std::lock_guard<std::mutex> g(s->mu);
      const Clock::time_point now = Clock::now();
      for (Job *j : batch) {
        j->finished = now;
        j->done = true;
        if (j->st != WL_OK) s->err = wl_last_error(ctx);
      }
      s->inflight -= est;
      if (s->inflight < 1.0) s->inflight = 0;
      s->running[lane] = 0;
      s->held[lane] = (double)wl_memory_held(ctx);
    }
    s->cvDone.notify_all();
    s->cvWork.notify_all();
  }
}

double ms(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

extern "C" {

void wl_serve_config_default(wl_serve_config *cfg) {
  if (!cfg) return;
  cfg->lanes = 2;
  cfg->memory_budget = (size_t)16 << 30;
  cfg->max_batch = 1024;
  cfg->stage_host_inputs = 1;
  cfg->max_batch_bytes = 0;
  cfg->express_lanes = 0;
  cfg->small_request_bytes = (size_t)4 << 20;
  cfg->express_priority = 0;
}

wl_status wl_serve_create(int device, const wl_serve_config *cfg, wl_server **out) {
  if (!out) return WL_EINVAL;
  *out = nullptr;
  wl_server *s = new wl_server;
  s->device = device;
  wl_serve_config_default(&s->cfg);
  if (cfg) s->cfg = *cfg;
  if (s->cfg.lanes < 1) s->cfg.lanes = 1;
  if (s->cfg.max_batch < 1) s->cfg.max_batch = 1;
  if (s->cfg.express_lanes < 0) s->cfg.express_lanes = 0;
  if (s->cfg.express_lanes >= s->cfg.lanes) s->cfg.express_lanes = s->cfg.lanes - 1;
  s->held.assign(s->cfg.lanes, 0.0);
  s->running.assign(s->cfg.lanes, 0.0);
  for (int i = 0; i < s->cfg.lanes; i++) {
    wl_ctx *c = nullptr;
    const wl_status st = wl_init(device, &c);
    if (st != WL_OK) {
      for (wl_ctx *x : s->ctxs) wl_destroy(x);
      delete s;
      return st;
    }
    s->ctxs.push_back(c);
    wl_set_host_input_mode(c, s->cfg.stage_host_inputs ? 1 : 0);
    if (i < s->cfg.express_lanes && s->cfg.express_priority) wl_set_stream_priority(c, 1);
  }
  for (int i = 0; i < s->cfg.lanes; i++) s->workers.emplace_back(worker, s, i);
  *out = s;
  return WL_OK;
}

wl_status wl_serve_submit_batch(wl_server *s, const wl_request *reqs, int n,
                                unsigned long long *tickets) {
  if (!s || !reqs || !tickets || n < 0) return WL_EINVAL;
  for (int i = 0; i < n; i++) {
    const wl_request *req = reqs + i;
    if (req->kind == WL_REQ_COMPRESS) {
      if (!req->cubelet.data)
        return serve_fail(s, WL_EINVAL, "request %d: compress request without data", i);
      for (int a = 0; a < 3; a++)
        if (req->cubelet.size[a] < 1)
          return serve_fail(s, WL_EINVAL, "request %d: empty cubelet size", i);
    } else if (req->kind == WL_REQ_DECOMPRESS) {
      if (!req->compressed || !req->out)
        return serve_fail(s, WL_EINVAL, "request %d: decompress request without input or output",
                          i);
    } else {
      return serve_fail(s, WL_EINVAL, "request %d: unknown request kind %d", i, req->kind);
    }
  }
  std::vector<Job *> js(n);
  const Clock::time_point now = Clock::now();
  for (int i = 0; i < n; i++) {
    Job *j = new Job;
    j->req = reqs[i];
    memset(&j->res, 0, sizeof j->res);
    j->est = estimate(reqs[i]);
    j->bytes = request_bytes(reqs[i]);
    j->submitted = now;
    js[i] = j;
  }
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) {
      for (Job *j : js) delete j;
      return WL_EINVAL;
    }
    for (int i = 0; i < n; i++) {
      Job *j = js[i];
      j->id = s->nextId++;
      s->jobs[j->id] = j;
      s->pending.push_back(j);
      tickets[i] = j->id;
    }
  }
  // every lane: an express lane may not serve what was queued, another may
  s->cvWork.notify_all();
  return WL_OK;
}

wl_status wl_serve_submit(wl_server *s, const wl_request *req, unsigned long long *ticket) {
  return wl_serve_submit_batch(s, req, 1, ticket);
}

wl_status wl_serve_wait(wl_server *s, unsigned long long ticket, int timeout_ms, wl_result *out,
                        wl_request_info *info) {
  if (!s) return WL_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) {
    s->err = "unknown or already retired ticket";
    return WL_EINVAL;
  }
  Job *j = it->second;
  if (timeout_ms < 0) {
    s->cvDone.wait(lk, [&] { return j->done; });
  } else if (!j->done) {
    s->cvDone.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return j->done; });
  }
  if (!j->done) return WL_ETIMEOUT;
  s->jobs.erase(it);
  lk.unlock();
  if (info) {
    info->status = j->st;
    info->queue_ms = ms(j->submitted, j->started);
    info->service_ms = ms(j->started, j->finished);
    info->total_ms = ms(j->submitted, j->finished);
    info->batch_size = j->batchSize;
    info->lane = j->lane;
  }
  const wl_status st = j->st;
  if (j->req.kind == WL_REQ_COMPRESS) {
    if (out) *out = j->res;
    else wl_result_free(&j->res);
  }
  delete j;
  return st;
}

wl_status wl_serve_wait_batch(wl_server *s, const unsigned long long *tickets, int n,
                              wl_result *outs, wl_status *statuses) {
  if (!s || !tickets || n < 0) return WL_EINVAL;
  wl_status first = WL_OK;
  for (int i = 0; i < n; i++) {
    const wl_status st = wl_serve_wait(s, tickets[i], -1, outs ? outs + i : nullptr, nullptr);
    if (statuses) statuses[i] = st;
    if (st != WL_OK && first == WL_OK) first = st;
  }
  return first;
}

const char *wl_serve_last_error(const wl_server *s) {
  return s ? s->err.c_str() : "null server";
}

void wl_serve_destroy(wl_server *s) {
  if (!s) return;
  std::deque<Job *> dropped;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    dropped.swap(s->pending);
    for (Job *j : dropped) {
      j->st = WL_EINVAL;
      j->done = true;
    }
  }
  s->cvWork.notify_all();
  s->cvDone.notify_all();
  for (std::thread &t : s->workers) t.join();
  for (auto &kv : s->jobs) {
    if (kv.second->req.kind == WL_REQ_COMPRESS && kv.second->st == WL_OK)
      wl_result_free(&kv.second->res);
    delete kv.second;
  }
  for (wl_ctx *c : s->ctxs) wl_destroy(c);
  delete s;
}

}  // extern "C"
