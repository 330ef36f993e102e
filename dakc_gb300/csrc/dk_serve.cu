// Serving loop: continuous batching of counting jobs over several engine
// workers.  (DAKC has no serving path: each run counts one file,
// dakc/src/main/main.cpp:42-49.  This layer keeps contexts, partitions and
// tables resident on the device between jobs and coalesces waiting jobs.)
//
// Model:
//   * dk_submit enqueues a job (the text is borrowed until the job completes)
//     after admission: its device-memory estimate must fit one worker's share
//     of the budget, else DK_ERR_ADMISSION.
//   * Each worker thread owns an Engine (its own CUDA stream and arenas).
//     Whenever a worker is idle it takes every queued job that fits its share
//     of the budget (same line width / k / variant, at most max_batch jobs)
//     and counts them with one dk_count_batch pipeline.  Jobs that arrive
//     while other workers run are picked up by the next free worker, so their
//     work overlaps on the device.
//   * dk_poll / dk_wait return the job's table -- host-resident, or left in
//     device memory when the job's descriptor asks for device residency (then
//     it stays valid until dk_serve_stop); dk_table_free releases it.  Waits
//     are bounded by the caller's timeout.
#include "dk_engine.hpp"
#include "../../include/dakc_gb300.h"

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace dk {

namespace {
using Clock = std::chrono::steady_clock;
double us_since(Clock::time_point t0, Clock::time_point t) {
  return std::chrono::duration<double, std::micro>(t - t0).count();
}
}  // namespace

struct Request {
  uint64_t ticket = 0;
  const char* text = nullptr;
  uint64_t nbytes = 0;
  dk_input_desc desc{};
  uint64_t est = 0;
  uint64_t kmers = 0;  // upper bound: lines * (line_width - k + 1)
  Clock::time_point t_submit, t_start, t_end;
  int status = DK_ERR_PENDING;
  // cancelled while its batch runs: it stays pending (its text is still
  // read) until the batch ends, then becomes DK_ERR_CANCELLED
  bool cancel = false;
  dk_table table{};
  int worker = -1;
  int batch_jobs = 0;
};

struct Worker {
  std::unique_ptr<Engine> eng;
  std::thread th;
  uint64_t budget = 0;
};

struct Server {
  // k-mers (upper bound) a worker gathers into one batch: about 5 ms of
  // device time -- enough to amortise a batch's fixed costs, short enough
  // that small jobs are not held behind large ones
  static constexpr uint64_t kBatchKmers = 128ull << 20;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> jobs;
  std::vector<Worker> workers;
  std::atomic<bool> stop{false};
  uint64_t next_ticket = 1;
  int max_batch = 1024;
  Clock::time_point t0 = Clock::now();
  uint64_t batches = 0, batched_jobs = 0;

  static uint64_t estimate(const dk_input_desc& d, uint64_t nbytes) {
    const uint64_t stride = (uint64_t)d.line_width + 1;
    const uint64_t lines = (nbytes + 1) / stride;
    const uint64_t per = d.line_width >= d.k ? (uint64_t)(d.line_width - d.k + 1) : 0;
    return lines * stride + 32 * lines * per + (1u << 20);
  }

  void run_worker(int w) {
    Worker& me = workers[w];
    for (;;) {
      std::vector<std::shared_ptr<Request>> batch;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop.load() || !queue.empty(); });
        if (stop.load() && queue.empty()) return;
        // coalesce queued jobs that fit this worker's share of the budget, up
        // to about kBatchKmers k-mers: a larger queue is left to the other
        // workers, so that batches run side by side and latency stays bounded
        const dk_input_desc d0 = queue.front()->desc;
        uint64_t bytes = 0, kmers = 0;
        for (auto it = queue.begin();
             it != queue.end() && (int)batch.size() < max_batch && kmers < kBatchKmers;) {
          const auto& r = *it;
          const bool same = r->desc.line_width == d0.line_width && r->desc.k == d0.k &&
                            r->desc.variant == d0.variant &&
                            r->desc.residency == d0.residency;
          if (same && (batch.empty() || bytes + r->est <= (uint64_t)(0.7 * (double)me.budget))) {
            bytes += r->est;
            kmers += r->kmers;
            batch.push_back(r);
            it = queue.erase(it);
          } else {
            ++it;
          }
        }
        const auto now = Clock::now();
        for (auto& r : batch) { r->t_start = now; r->worker = w; }
      }
      std::vector<dk_job> jv(batch.size());
      std::vector<dk_table> outs(batch.size());
      for (size_t i = 0; i < batch.size(); ++i) jv[i] = {batch[i]->text, batch[i]->nbytes};
      dk_input_desc d = batch[0]->desc;  // host or device tables, as the jobs asked
      const int rc = me.eng->count_batch(jv.data(), (int)jv.size(), &d, outs.data());
      {
        std::lock_guard<std::mutex> lk(mu);
        const auto now = Clock::now();
        ++batches;
        batched_jobs += batch.size();
        for (size_t i = 0; i < batch.size(); ++i) {
          auto& r = batch[i];
          r->t_end = now;
          r->batch_jobs = (int)batch.size();
          if (r->cancel) {
            if (rc == DK_OK) me.eng->release_table(outs[i].handle);
            r->status = DK_ERR_CANCELLED;  // dk_poll reports it; the text is free
            continue;
          }
          r->status = rc;
          if (rc == DK_OK) {
            r->table = outs[i];
            // tag the handle with its worker so dk_table_free finds the pool
            r->table.handle = outs[i].handle | ((uint64_t)(w + 1) << 48);
          }
        }
      }
      cv_done.notify_all();
    }
  }
};

}  // namespace dk

using dk::Server;

// The serving state hangs off the context created by dk_create.
namespace dk {
Server* server_of(dk_ctx* ctx);
void set_server(dk_ctx* ctx, Server* s);
Engine* engine_of(dk_ctx* ctx);
int serve_release(Server* s, uint64_t handle);
}  // namespace dk

extern "C" {

int dk_serve_start(dk_ctx* ctx, int workers, int max_batch_jobs) {
  if (!ctx || workers < 1 || workers > 16 || max_batch_jobs < 1) return DK_ERR_INVALID_ARG;
  if (dk::server_of(ctx)) return DK_ERR_INVALID_ARG;
  dk::Engine* base = dk::engine_of(ctx);
  auto* s = new (std::nothrow) Server();
  if (!s) return DK_ERR_OOM;
  s->max_batch = std::min(max_batch_jobs, 4096);
  const uint64_t share = base->budget / (uint64_t)workers;
  s->workers.resize(workers);
  for (int w = 0; w < workers; ++w) {
    s->workers[w].eng.reset(new dk::Engine());
    dk_config cfg{};
    cfg.device = base->device;
    cfg.mem_budget = share;
    cfg.flags = base->flags;  // workers count as the context would
    const int rc = s->workers[w].eng->init(&cfg);
    if (rc != DK_OK) {
      delete s;
      return rc;
    }
    s->workers[w].budget = share;
    // host tables come from (and return to) the context's pool, so a table
    // size any worker has used is ready for every worker
    s->workers[w].eng->hpool = base->hpool;
  }
  for (int w = 0; w < workers; ++w) s->workers[w].th = std::thread([s, w] { s->run_worker(w); });
  dk::set_server(ctx, s);
  return DK_OK;
}

int dk_submit(dk_ctx* ctx, const char* text, uint64_t nbytes, const dk_input_desc* desc,
              uint64_t* ticket) {
  Server* s = ctx ? dk::server_of(ctx) : nullptr;
  if (!s || !desc || !ticket || (!text && nbytes)) return DK_ERR_INVALID_ARG;
  if (desc->k < 1 || desc->k > 32 || desc->line_width < 1 || desc->line_width > 1024 ||
      !dk::convention_ok(*desc) || dk::frame_lines(nbytes, desc->line_width) < 0)
    return DK_ERR_INVALID_ARG;
  auto r = std::make_shared<dk::Request>();
  r->text = text;
  r->nbytes = nbytes;
  r->desc = *desc;
  r->est = Server::estimate(*desc, nbytes);
  {
    const uint64_t lines = (nbytes + desc->line_width) / ((uint64_t)desc->line_width + 1);
    r->kmers = lines * (desc->line_width >= desc->k ? (uint64_t)(desc->line_width - desc->k + 1) : 0);
  }
  if (r->est > (uint64_t)(0.7 * (double)s->workers[0].budget)) return DK_ERR_ADMISSION;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->next_ticket++;
    r->t_submit = dk::Clock::now();
    s->jobs[r->ticket] = r;
    s->queue.push_back(r);
  }
  s->cv_work.notify_one();
  *ticket = r->ticket;
  return DK_OK;
}

static int take_result(Server* s, uint64_t ticket, dk_table* out, dk_job_info* info) {
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return DK_ERR_NOT_FOUND;
  auto r = it->second;
  if (r->status == DK_ERR_PENDING) return DK_ERR_PENDING;
  const int st = r->status;
  if (out) {
    *out = r->table;
  } else if (st == DK_OK && r->table.handle) {
    dk::serve_release(s, r->table.handle);  // no one takes the table: free it now
  }
  if (info) {
    info->queued_us = dk::us_since(r->t_submit, r->t_start);
    info->run_us = dk::us_since(r->t_start, r->t_end);
    info->batch_jobs = r->batch_jobs;
    info->worker = r->worker;
  }
  s->jobs.erase(it);
  return st;
}

int dk_poll(dk_ctx* ctx, uint64_t ticket, dk_table* out, dk_job_info* info) {
  Server* s = ctx ? dk::server_of(ctx) : nullptr;
  if (!s) return DK_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  return take_result(s, ticket, out, info);
}

int dk_wait(dk_ctx* ctx, uint64_t ticket, int timeout_ms, dk_table* out, dk_job_info* info) {
  Server* s = ctx ? dk::server_of(ctx) : nullptr;
  if (!s) return DK_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto deadline = dk::Clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
  for (;;) {
    const int st = take_result(s, ticket, out, info);
    if (st != DK_ERR_PENDING) return st;
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) {
      const int st2 = take_result(s, ticket, out, info);
      return st2 == DK_ERR_PENDING ? DK_ERR_TIMEOUT : st2;
    }
  }
}

int dk_cancel(dk_ctx* ctx, uint64_t ticket) {
  Server* s = ctx ? dk::server_of(ctx) : nullptr;
  if (!s) return DK_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return DK_ERR_NOT_FOUND;
  auto r = it->second;
  for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
    if ((*q)->ticket == ticket) {
      s->queue.erase(q);
      r->status = DK_ERR_CANCELLED;
      s->cv_done.notify_all();  // a dk_wait on this ticket returns now
      return DK_OK;
    }
  if (r->status == DK_ERR_PENDING) {  // running: its table is dropped when the batch ends
    r->cancel = true;
    return DK_OK;
  }
  return DK_ERR_INVALID_ARG;  // already finished: take it with dk_poll and free it
}

int dk_serve_stop(dk_ctx* ctx) {
  Server* s = ctx ? dk::server_of(ctx) : nullptr;
  if (!s) return DK_ERR_INVALID_ARG;
  {
    // under the lock: a worker between its wait predicate and its sleep
    // would otherwise miss the notification and never wake
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop.store(true);
  }
  s->cv_work.notify_all();
  for (auto& w : s->workers)
    if (w.th.joinable()) w.th.join();
  // finished jobs whose tables nobody took go back to the pool
  for (auto& kv : s->jobs) {
    dk::Request& r = *kv.second;
    if (r.status == DK_OK && r.table.handle) dk::serve_release(s, r.table.handle);
  }
  s->jobs.clear();
  dk::set_server(ctx, nullptr);
  delete s;
  return DK_OK;
}

}  // extern "C"

namespace dk {
// release a served table (handle tagged with its worker)
int serve_release(Server* s, uint64_t handle) {
  const int w = (int)(handle >> 48) - 1;
  if (!s || w < 0 || w >= (int)s->workers.size()) return DK_ERR_NOT_FOUND;
  Engine* e = s->workers[w].eng.get();
  return e->release_table(handle & ((1ull << 48) - 1));  // the pool has its own lock
}
}  // namespace dk
