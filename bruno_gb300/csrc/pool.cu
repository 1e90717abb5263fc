/*
 * pool.cu -- many graph builds on one GPU at once: a pool of worker threads, each owning one
 * context (its own stream and buffers), runs bruno_build_and_compact for queued requests.
 *
 * The reference builds one graph per MPI job.  On one GB300 a small graph (a few Mbp) leaves
 * most of the GPU idle, and one build issues several dozen short kernels and a dozen
 * host round trips; running builds side by side on separate streams fills the GPU with the
 * kernels of several builds at once.  Two forms sit on top of this pool:
 *   - batched: submit a whole set of samples, then wait for all of them;
 *   - served:  submit requests as they arrive; each is admitted to a worker as soon as one is
 *              free and its device-memory estimate fits the pool's budget, so requests that
 *              arrive while others run overlap with them on the device.
 * Every build runs the plain path unchanged, in its own context, so its outputs are the
 * plain path's outputs bit for bit, alone or in any mix.
 *
 * Admission: a worker keeps its context's buffers between requests, so the pool tracks per
 * worker the largest estimate it has run (what its buffers may hold) and admits the request at
 * the head of the queue to a free worker only while the sum over workers stays within the
 * budget -- or when no other worker is busy, so that a request larger than the budget still
 * runs alone.  The estimate is 20 bytes of device memory per FASTQ byte plus 64 MiB.  When the
 * request at the head of the queue fits nowhere, idle workers free their buffers; a request
 * that still runs out of device memory is queued again, once, to run with no other build busy,
 * and no other request starts until it has finished.
 *
 * The batched mode (bruno_pool_create_batched) replaces the workers by two schedulers that run
 * continuous batching over the fused form: every pass takes the queued requests that fit its
 * scheduler's share of the budget and builds them together in one pass of every kernel
 * (bruno_build_samples).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <set>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/bruno_gb300.h"
#include "pool_admission.h"

namespace {

using clk = std::chrono::steady_clock;

struct Request {
  uint64_t ticket;
  const char *buf;
  size_t n;
  uint64_t est;
  clk::time_point submitted;
  bool solo;   /* ran out of memory beside others once: now runs with no other build busy */
};

struct Done {
  bruno_pool_result r;
};

}  // namespace

struct bruno_pool {
  bruno_cfg cfg{};
  uint64_t budget = 0;
  bool batched = false;          /* continuous batching: scheduler threads running fused passes */
  uint32_t max_samples = 0;      /* requests in one fused pass at most */
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request> queue;
  std::map<uint64_t, Done> done;
  std::vector<std::thread> threads;
  std::vector<uint64_t> held;    /* per worker: largest estimate run so far */
  std::vector<bool> busy;
  bool solo_running = false;     /* a retried request is running and must stay alone */
  std::set<uint64_t> collected;  /* tickets whose results were already handed out */
  uint64_t next_ticket = 1;
  bool stop = false;
};

namespace {

using bruno_pool_rules::estimate;

/* may worker w take request q now?  (called with the lock held) */
bool admits(const bruno_pool *p, int w, const Request &q) {
  return bruno_pool_rules::admits(p->held, p->busy, p->budget, w, q.est, q.solo, p->solo_running);
}

/* should idle worker w free its buffers so that the queue head fits?  (lock held) */
bool should_trim(const bruno_pool *p, int w) {
  if (p->queue.empty()) return false;
  const Request &q = p->queue.front();
  return bruno_pool_rules::should_trim(p->held, p->busy, p->budget, w, q.est, q.solo, p->solo_running);
}

void run_one(bruno_ctx *ctx, int words, const Request &q, bruno_pool_result &r) {
  r.words = words;
  r.status = bruno_build_and_compact(ctx, q.buf, q.n, 0);
  if (r.status == BRUNO_OK) r.status = bruno_get_sizes(ctx, &r.sizes);
  if (r.status != BRUNO_OK) return;
  size_t nc = 0, nch = 0;
  r.status = bruno_copy_chains(ctx, nullptr, nullptr, nullptr, 0, 0, &nc, &nch);
  if (r.status != BRUNO_OK) return;
  r.reps = (uint64_t *)std::malloc(std::max<size_t>(1, nc) * 8 * words);
  r.offsets = (uint64_t *)std::malloc((nc + 1) * 8);
  r.chars = (char *)std::malloc(std::max<size_t>(1, nch));
  if (!r.reps || !r.offsets || !r.chars) { r.status = BRUNO_ERR_OOM; return; }
  r.status = bruno_copy_chains(ctx, r.reps, r.offsets, r.chars, nc, nch, &nc, &nch);
  r.n_chains = nc;
  r.n_chars = nch;
}

void worker_main(bruno_pool *p, int w) {
  bruno_ctx *ctx = nullptr;
  for (;;) {
    Request q;
    {
      std::unique_lock<std::mutex> lk(p->mu);
      p->cv_work.wait(lk, [&] {
        return p->stop || (!p->queue.empty() && (admits(p, w, p->queue.front()) || should_trim(p, w)));
      });
      if (p->stop && p->queue.empty()) break;
      if (should_trim(p, w)) {   /* free this worker's buffers for the request at the head */
        lk.unlock();
        if (ctx) { bruno_ctx_destroy(ctx); ctx = nullptr; }
        lk.lock();
        p->held[w] = 0;
        lk.unlock();
        p->cv_work.notify_all();
        continue;
      }
      if (p->queue.empty() || !admits(p, w, p->queue.front())) continue;
      q = p->queue.front();
      p->queue.pop_front();
      p->busy[w] = true;
      p->held[w] = std::max(p->held[w], q.est);
      if (q.solo) p->solo_running = true;
    }
    const clk::time_point t0 = clk::now();
    Done d;
    std::memset(&d.r, 0, sizeof(d.r));
    const bruno_status cst = ctx ? BRUNO_OK : bruno_ctx_create(&p->cfg, &ctx);
    if (cst != BRUNO_OK) d.r.status = cst;
    else run_one(ctx, p->cfg.k <= 31 ? 1 : 2, q, d.r);
    /* out of device memory: free this worker's buffers before anything else */
    const bool trim = d.r.status == BRUNO_ERR_OOM;
    if (trim && ctx) { bruno_ctx_destroy(ctx); ctx = nullptr; }
    if (d.r.status == BRUNO_ERR_OOM && !q.solo) {   /* once more, with no other build beside it */
      bruno_pool_result_free(&d.r);
      {
        std::lock_guard<std::mutex> lk(p->mu);
        p->busy[w] = false;
        p->held[w] = 0;
        q.solo = true;   /* solo_running is still false: this request was not solo */
        p->queue.push_front(q);
      }
      p->cv_work.notify_all();
      continue;
    }
    const clk::time_point t1 = clk::now();
    d.r.queue_ms = std::chrono::duration<double, std::milli>(t0 - q.submitted).count();
    d.r.run_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    d.r.worker = w;
    {
      std::lock_guard<std::mutex> lk(p->mu);
      p->busy[w] = false;
      if (q.solo) p->solo_running = false;
      if (trim) p->held[w] = 0;
      p->done[q.ticket] = d;
    }
    p->cv_done.notify_all();
    p->cv_work.notify_all();   /* memory held by this worker may now admit the queue head */
  }
  if (ctx) bruno_ctx_destroy(ctx);
}

/* copies one sample's results of a fused pass into a result record */
void take_sample(bruno_ctx *ctx, size_t i, int words, bruno_pool_result &r) {
  r.words = words;
  r.status = bruno_sample_sizes(ctx, i, &r.sizes);
  if (r.status != BRUNO_OK) return;
  size_t nc = 0, nch = 0;
  r.status = bruno_sample_copy_chains(ctx, i, nullptr, nullptr, nullptr, 0, 0, &nc, &nch);
  if (r.status != BRUNO_OK) return;
  r.reps = (uint64_t *)std::malloc(std::max<size_t>(1, nc) * 8 * words);
  r.offsets = (uint64_t *)std::malloc((nc + 1) * 8);
  r.chars = (char *)std::malloc(std::max<size_t>(1, nch));
  if (!r.reps || !r.offsets || !r.chars) { r.status = BRUNO_ERR_OOM; return; }
  r.status = bruno_sample_copy_chains(ctx, i, r.reps, r.offsets, r.chars, nc, nch, &nc, &nch);
  r.n_chains = nc;
  r.n_chars = nch;
}

/* Continuous batching: a scheduler takes every queued request that fits its share of the memory
 * budget (at least one, at most max_samples), builds them in one fused pass (bruno_build_samples),
 * and hands out each request's results; requests that arrive during a pass wait for the next one.
 * Where the fused pass cannot run (a configuration the batched form refuses, or an error), each
 * request of the pass is built on its own with the plain path, so every result is always the
 * plain path's.  Scheduler w has its own context; with two schedulers one pass's host work (the
 * copies in, every request's results out) runs beside the other pass's kernels. */
void batch_main(bruno_pool *p, int w) {
  bruno_ctx *ctx = nullptr;
  const int words = p->cfg.k <= 31 ? 1 : 2;
  const uint64_t share = p->budget / p->held.size();
  for (;;) {
    std::vector<Request> take;
    {
      std::unique_lock<std::mutex> lk(p->mu);
      p->cv_work.wait(lk, [&] { return p->stop || !p->queue.empty(); });
      if (p->stop && p->queue.empty()) break;
      uint64_t sum = 0;
      while (!p->queue.empty() && take.size() < p->max_samples) {
        const Request &q = p->queue.front();
        if (!take.empty() && sum + q.est > share) break;
        sum += q.est;
        take.push_back(q);
        p->queue.pop_front();
      }
      p->busy[w] = true;
      p->held[w] = std::max(p->held[w], sum);
    }
    const clk::time_point t0 = clk::now();
    std::vector<Done> out(take.size());
    for (auto &d : out) std::memset(&d.r, 0, sizeof(d.r));
    bruno_status st = ctx ? BRUNO_OK : bruno_ctx_create(&p->cfg, &ctx);
    if (st == BRUNO_OK) {
      std::vector<const char *> bufs(take.size());
      std::vector<size_t> ns(take.size());
      for (size_t i = 0; i < take.size(); ++i) { bufs[i] = take[i].buf; ns[i] = take[i].n; }
      st = take.size() > 1 ? bruno_build_samples(ctx, bufs.data(), ns.data(), take.size(), 0) : BRUNO_ERR_ARG;
      if (st == BRUNO_OK) {
        for (size_t i = 0; i < take.size(); ++i) take_sample(ctx, i, words, out[i].r);
      } else {   /* one request, or a pass the batched form cannot take: the plain path, one by one */
        for (size_t i = 0; i < take.size(); ++i) run_one(ctx, words, take[i], out[i].r);
      }
    } else {
      for (auto &d : out) d.r.status = st;
    }
    const clk::time_point t1 = clk::now();
    {
      std::lock_guard<std::mutex> lk(p->mu);
      for (size_t i = 0; i < take.size(); ++i) {
        out[i].r.queue_ms = std::chrono::duration<double, std::milli>(t0 - take[i].submitted).count();
        out[i].r.run_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        out[i].r.worker = w;
        p->done[take[i].ticket] = out[i];
      }
      p->busy[w] = false;
    }
    p->cv_done.notify_all();
  }
  if (ctx) bruno_ctx_destroy(ctx);
}

}  // namespace

extern "C" bruno_status bruno_pool_create_batched(const bruno_cfg *cfg, uint32_t max_samples, uint64_t mem_budget,
                                                  bruno_pool **out) {
  if (!cfg || !out || max_samples < 1 || max_samples > 16384) return BRUNO_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(cfg->device) != cudaSuccess) { cudaGetLastError(); return BRUNO_ERR_CUDA; }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) { cudaGetLastError(); return BRUNO_ERR_CUDA; }
  bruno_pool *p = new bruno_pool();
  p->cfg = *cfg;
  p->batched = true;
  p->max_samples = max_samples;
  p->budget = mem_budget ? mem_budget : (uint64_t)(0.8 * (double)free_b);
  constexpr int SCHEDULERS = 2;
  p->held.assign(SCHEDULERS, 0);
  p->busy.assign(SCHEDULERS, false);
  for (int w = 0; w < SCHEDULERS; ++w) p->threads.emplace_back(batch_main, p, w);
  *out = p;
  return BRUNO_OK;
}

extern "C" bruno_status bruno_pool_create(const bruno_cfg *cfg, int32_t workers, uint64_t mem_budget,
                                          bruno_pool **out) {
  if (!cfg || !out || workers < 1 || workers > 256) return BRUNO_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(cfg->device) != cudaSuccess) { cudaGetLastError(); return BRUNO_ERR_CUDA; }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) { cudaGetLastError(); return BRUNO_ERR_CUDA; }
  bruno_pool *p = new bruno_pool();
  p->cfg = *cfg;
  p->budget = mem_budget ? mem_budget : (uint64_t)(0.8 * (double)free_b);
  p->held.assign(workers, 0);
  p->busy.assign(workers, false);
  for (int w = 0; w < workers; ++w) p->threads.emplace_back(worker_main, p, w);
  *out = p;
  return BRUNO_OK;
}

extern "C" bruno_status bruno_pool_submit(bruno_pool *p, const char *buf, size_t nbytes, uint64_t *ticket) {
  if (!p || !ticket || (!buf && nbytes)) return BRUNO_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(p->mu);
    if (p->stop) return BRUNO_ERR_ARG;
    *ticket = p->next_ticket++;
    p->queue.push_back(Request{*ticket, buf, nbytes, estimate(nbytes), clk::now(), false});
  }
  p->cv_work.notify_all();
  return BRUNO_OK;
}

extern "C" bruno_status bruno_pool_wait(bruno_pool *p, uint64_t ticket, bruno_pool_result *out) {
  if (!p || !out) return BRUNO_ERR_ARG;
  std::unique_lock<std::mutex> lk(p->mu);
  if (ticket == 0 || ticket >= p->next_ticket || p->collected.count(ticket)) return BRUNO_ERR_ARG;
  p->collected.insert(ticket);   /* a second wait on this ticket is an error, not a hang */
  p->cv_done.wait(lk, [&] { return p->done.count(ticket) != 0; });
  *out = p->done[ticket].r;
  p->done.erase(ticket);
  return BRUNO_OK;
}

extern "C" bruno_status bruno_pool_result_free(bruno_pool_result *r) {
  if (!r) return BRUNO_ERR_ARG;
  std::free(r->reps); std::free(r->offsets); std::free(r->chars);
  r->reps = nullptr; r->offsets = nullptr; r->chars = nullptr;
  return BRUNO_OK;
}

extern "C" bruno_status bruno_pool_destroy(bruno_pool *p) {
  if (!p) return BRUNO_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(p->mu);
    p->stop = true;
  }
  p->cv_work.notify_all();
  for (auto &t : p->threads) t.join();
  for (auto &kv : p->done) bruno_pool_result_free(&kv.second.r);
  delete p;
  return BRUNO_OK;
}
