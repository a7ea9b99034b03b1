// Request server: continuous batching of SCAN queries and new-graph counts on
// one GPU.
//
// Design: `workers` host threads, each with its own non-blocking CUDA stream
// and its own query context on the resident graph.  A shared queue holds
// requests in arrival order; an idle worker takes the first request whose
// admission size fits the remaining HBM budget (first fit, so a small request is
// not held behind a large one that must wait for memory), reserves the bytes,
// runs it on its stream, releases the bytes and publishes the result.  Requests
// therefore start the moment a worker and memory are free, and the kernels of
// concurrent requests overlap on the device.  Results are exact: a query's
// digest and counts do not depend on what else runs (the resident graph is only
// read; every request owns its scratch).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "accx_internal.h"
#include "gen_host.h"

using sclock = std::chrono::steady_clock;

struct srv_req {
  uint64_t id;
  accx_request req;
  uint64_t bytes;
  sclock::time_point t_submit, t_start, t_done;
  bool done = false;
  accx_result res{};
};

struct accx_server {
  accx_graph *g = nullptr;
  accx_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<srv_req *> pending;
  std::unordered_map<uint64_t, srv_req *> all;
  std::vector<std::thread> threads;
  uint64_t next_id = 1, used = 0, peak = 0;
  int running = 0, max_running = 0;
  bool stop = false;
  uint64_t submitted = 0, completed = 0, failed = 0;
  sclock::time_point t0;
  bool started = false;
  int count_sms = 0;
  std::vector<double> lat_q, lat_c;
};

static double ms_between(sclock::time_point a, sclock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

extern "C" uint64_t accx_server_request_bytes(const accx_server *s, const accx_request *r) {
  if (!s || !r) return 0;
  if (r->type == ACCX_REQ_QUERY) return 0;  // queries use the worker's preallocated context
  uint32_t n = 0;
  uint64_t draws = 0;
  if (accx_gen_shape(&r->graph, &n, &draws) != ACCX_OK) return 0;
  // generation: 2 keys per draw x 8 bytes, sort double buffer + unique copy;
  // graph: offsets + entries; counting scratch: counts, owned-edge list,
  // per-vertex work and prefix arrays
  const uint64_t keys = 2 * draws;
  uint64_t b = 3 * 8 * keys + 4ull * (n + 1) + 4 * keys + 4 * keys + 8 * (keys / 2) + 40ull * (n + 1);
  // oriented counts: the relabeled copy (4(n+1) + 12m) and the oriented scratch
  // (prefix lengths, reverse entries, partner ranges, work items)
  if (s->cfg.count_orient) b += 4ull * (n + 1) + 12 * keys + 16 * keys + 12ull * (n + 1) + keys / 8;
  return b;
}

static void run_request(accx_server *S, srv_req *q, accx_query_ctx *ctx, cudaStream_t st_query,
                        cudaStream_t st) {
  accx_result &R = q->res;
  R.type = q->req.type;
  if (q->req.type == ACCX_REQ_QUERY) {
    R.status = accx_scan_query_ctx(S->g, ctx, q->req.eps, q->req.mu, nullptr, nullptr, nullptr, &R.summary, st_query);
    return;
  }
  accx_graph *h = nullptr;
  R.status = accx_graph_generate(&q->req.graph, st, &h);
  if (R.status) return;
  accx_count_opts o;
  memset(&o, 0, sizeof(o));
  o.policy = S->cfg.count_policy;
  o.sm_limit = S->count_sms;
  if (S->cfg.count_orient) {
    o.orient = 1;
    R.status = accx_graph_relabel(h, st);  // prefix lists are short only on the degree-ordered copy
  }
  if (!R.status) R.status = accx_cn_count(h, &o, nullptr, st);
  if (!R.status) R.status = accx_cn_digest(h, &R.count_sum, &R.count_digest, st);
  R.n = h->n;
  R.m = h->m;
  accx_graph_free(h);
}

static void worker(accx_server *S) {
  cudaSetDevice(S->g->device);
  // queries on the highest-priority stream, counts on the lowest: the block
  // scheduler then starts pending query blocks first
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  cudaStream_t st = nullptr, stq = nullptr;
  cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, lo);
  cudaStreamCreateWithPriority(&stq, cudaStreamNonBlocking, hi);
  accx_query_ctx *ctx = nullptr;
  int ctx_rc = accx_query_ctx_create(S->g, &ctx);
  for (;;) {
    srv_req *q = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      for (;;) {
        if (S->stop && S->pending.empty()) break;
        const uint64_t budget = S->cfg.hbm_budget;
        for (auto it = S->pending.begin(); it != S->pending.end(); ++it) {
          // first fit; a request larger than the whole budget runs alone
          if ((*it)->bytes <= budget - std::min(budget, S->used) || (S->used == 0 && (*it)->bytes > budget)) {
            q = *it;
            S->pending.erase(it);
            break;
          }
        }
        if (q) break;
        S->cv_work.wait(lk);
      }
      if (!q) break;
      S->used += q->bytes;
      S->peak = std::max(S->peak, S->used);
      S->running++;
      S->max_running = std::max(S->max_running, S->running);
      q->t_start = sclock::now();
    }
    if (q->req.type == ACCX_REQ_QUERY && ctx_rc) q->res.status = ctx_rc;
    else run_request(S, q, ctx, stq, st);
    {
      std::lock_guard<std::mutex> lk(S->mu);
      q->t_done = sclock::now();
      q->res.queue_ms = ms_between(q->t_submit, q->t_start);
      q->res.run_ms = ms_between(q->t_start, q->t_done);
      q->res.latency_ms = ms_between(q->t_submit, q->t_done);
      q->done = true;
      S->used -= q->bytes;
      S->running--;
      S->completed++;
      if (q->res.status) S->failed++;
      (q->req.type == ACCX_REQ_QUERY ? S->lat_q : S->lat_c).push_back(q->res.latency_ms);
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
  if (ctx) accx_query_ctx_free(ctx);
  cudaStreamDestroy(st);
  cudaStreamDestroy(stq);
}

extern "C" int accx_server_create(accx_graph *resident, const accx_server_config *cfg, accx_server **out) {
  if (!resident || !out) return ACCX_ERR_INVALID_ARG;
  if (!resident->cnt_valid) return ACCX_ERR_NOT_READY;
  if (cfg && cfg->count_policy == ACCX_POLICY_TABLE) return ACCX_ERR_INVALID_ARG;
  // the workers' streams do not wait on other streams: finish everything already
  // queued (the resident graph's count among it) before they start reading it
  ACCX_CUDA_TRY(cudaSetDevice(resident->device));
  ACCX_CUDA_TRY(cudaDeviceSynchronize());
  accx_server *S = new (std::nothrow) accx_server();
  if (!S) return ACCX_ERR_OOM;
  S->g = resident;
  if (cfg) S->cfg = *cfg;
  if (S->cfg.workers <= 0) S->cfg.workers = 4;
  if (S->cfg.workers > 64) S->cfg.workers = 64;
  if (S->cfg.hbm_budget == 0) S->cfg.hbm_budget = 64ull << 30;
  if (S->cfg.count_sm_percent <= 0 || S->cfg.count_sm_percent > 100) S->cfg.count_sm_percent = 50;
  S->count_sms = accx_sm_count(resident->device) * S->cfg.count_sm_percent / 100;
  if (S->count_sms < 1) S->count_sms = 1;
  for (int i = 0; i < S->cfg.workers; i++) S->threads.emplace_back(worker, S);
  *out = S;
  return ACCX_OK;
}

extern "C" int accx_server_submit(accx_server *S, const accx_request *r, uint64_t *id) {
  if (!S || !r) return ACCX_ERR_INVALID_ARG;
  if (r->type != ACCX_REQ_QUERY && r->type != ACCX_REQ_COUNT) return ACCX_ERR_INVALID_ARG;
  if (r->type == ACCX_REQ_COUNT) {
    uint32_t n;
    uint64_t draws;
    int rc = accx_gen_shape(&r->graph, &n, &draws);
    if (rc) return rc;
  }
  srv_req *q = new (std::nothrow) srv_req();
  if (!q) return ACCX_ERR_OOM;
  q->req = *r;
  q->bytes = accx_server_request_bytes(S, r);
  q->t_submit = sclock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) {
      delete q;
      return ACCX_ERR_INVALID_ARG;
    }
    if (!S->started) {
      S->started = true;
      S->t0 = q->t_submit;
    }
    q->id = S->next_id++;
    S->all[q->id] = q;
    S->pending.push_back(q);
    S->submitted++;
    if (id) *id = q->id;
  }
  S->cv_work.notify_one();
  return ACCX_OK;
}

extern "C" int accx_server_poll(accx_server *S, uint64_t id, accx_result *out) {
  if (!S) return ACCX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->all.find(id);
  if (it == S->all.end()) return ACCX_ERR_INVALID_ARG;
  if (!it->second->done) return ACCX_ERR_NOT_READY;
  if (out) *out = it->second->res;
  return ACCX_OK;
}

extern "C" int accx_server_wait(accx_server *S, uint64_t id, double timeout_ms, accx_result *out) {
  if (!S) return ACCX_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->all.find(id);
  if (it == S->all.end()) return ACCX_ERR_INVALID_ARG;
  srv_req *q = it->second;
  auto pred = [&] { return q->done; };
  if (timeout_ms < 0) S->cv_done.wait(lk, pred);
  else if (!S->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), pred))
    return ACCX_ERR_TIMEOUT;
  if (out) *out = q->res;
  return ACCX_OK;
}

extern "C" int accx_server_drain(accx_server *S) {
  if (!S) return ACCX_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  S->cv_done.wait(lk, [&] { return S->completed == S->submitted; });
  return ACCX_OK;
}

static double pct(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  size_t i = (size_t)llround(p * (double)(v.size() - 1));
  return v[std::min(i, v.size() - 1)];
}

extern "C" int accx_server_stats_get(accx_server *S, accx_server_stats *o) {
  if (!S || !o) return ACCX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  memset(o, 0, sizeof(*o));
  o->submitted = S->submitted;
  o->completed = S->completed;
  o->failed = S->failed;
  o->query_p50_ms = pct(S->lat_q, 0.50);
  o->query_p99_ms = pct(S->lat_q, 0.99);
  o->count_p50_ms = pct(S->lat_c, 0.50);
  o->count_p99_ms = pct(S->lat_c, 0.99);
  sclock::time_point last = S->t0;
  for (auto &kv : S->all)
    if (kv.second->done && kv.second->t_done > last) last = kv.second->t_done;
  o->elapsed_s = S->started ? ms_between(S->t0, last) / 1e3 : 0.0;
  o->throughput_rps = o->elapsed_s > 0 ? (double)S->completed / o->elapsed_s : 0.0;
  o->max_concurrent = S->max_running;
  o->peak_bytes = S->peak;
  return ACCX_OK;
}

extern "C" int accx_server_destroy(accx_server *S) {
  if (!S) return ACCX_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto &t : S->threads) t.join();
  for (auto &kv : S->all) delete kv.second;
  delete S;
  return ACCX_OK;
}
