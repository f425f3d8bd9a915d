// Batched and served proving: a pool of prover contexts fed by a FIFO queue
// with HBM-footprint admission (include/z0p_gpu.h, "batching / serving").
//
// Each worker thread owns one context (its own CUDA stream and workspace),
// so independent proofs overlap on the GPU: one proof's kernels fill the
// SMs while another waits on its Fiat-Shamir round trip. Admission keeps the
// sum of running jobs' device footprints within the budget; the queue is
// strictly FIFO so a large job is never starved by smaller ones behind it.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/z0p_gpu.h"
#include "host.h"

namespace {

constexpr size_t kKeepBytes = 512ull << 20;  // workspace an idle worker may keep

struct Pending {
  z0p_job* job;
  uint64_t ticket;
  size_t footprint;
};

}  // namespace

struct z0p_gpu_pool {
  int device = 0;
  std::vector<z0p_gpu_ctx*> ctxs;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  std::deque<Pending> queue;
  std::unordered_map<uint64_t, int> done;
  size_t budget = 0, inflight = 0;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

int footprint(const z0p_job* j, size_t* bytes) {
  if (j->kind == Z0P_JOB_AIR) return z0p_gpu_air_footprint(&j->air, bytes);
  if (j->kind == Z0P_JOB_RANGE) return z0p_gpu_range_footprint(&j->range, bytes);
  return Z0P_ERR_INVALID_ARGUMENT;
}

void worker(z0p_gpu_pool* p, z0p_gpu_ctx* ctx) {
  cudaSetDevice(p->device);
  for (;;) {
    Pending item;
    {
      std::unique_lock<std::mutex> lk(p->mu);
      // FIFO head only, admitted when it fits next to the running jobs.
      p->work_cv.wait(lk, [&] {
        return p->stop ||
               (!p->queue.empty() && p->inflight + p->queue.front().footprint <= p->budget);
      });
      if (p->stop) return;
      item = p->queue.front();
      p->queue.pop_front();
      p->inflight += item.footprint;
      item.job->start_s = p->now();
    }
    // The next head may fit too.
    p->work_cv.notify_all();
    z0p_job* j = item.job;
    int rc;
    if (j->kind == Z0P_JOB_AIR)
      rc = z0p_gpu_air_prove(ctx, &j->air, j->transcript, j->out, j->cap, &j->len);
    else
      rc = z0p_gpu_range_prove(ctx, &j->range, j->transcript, j->out, j->cap, &j->len);
    // A context that just held a large job gives its workspace back to the
    // device pool, so memory held by idle workers stays small next to the
    // admission budget.
    if (z0p_gpu_ctx_device_bytes(ctx) > kKeepBytes) z0p_gpu_ctx_trim(ctx);
    {
      std::lock_guard<std::mutex> lk(p->mu);
      j->status = rc;
      j->end_s = p->now();
      p->inflight -= item.footprint;
      p->done[item.ticket] = rc;
    }
    p->done_cv.notify_all();
    p->work_cv.notify_all();
  }
}

}  // namespace

extern "C" {

int z0p_gpu_pool_create(int device, int workers, size_t hbm_budget, z0p_gpu_pool** out) {
  if (!out || workers < 1 || workers > 256) return Z0P_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  z0p_gpu_pool* p = new z0p_gpu_pool();
  p->device = device;
  if (hbm_budget == 0) {
    size_t free_b = 0, total_b = 0;
    cudaSetDevice(device);
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      delete p;
      z0p::host::set_reason("cudaMemGetInfo failed while sizing the pool budget");
      return Z0P_ERR_CUDA;
    }
    hbm_budget = free_b / 10 * 9;
  }
  p->budget = hbm_budget;
  for (int i = 0; i < workers; i++) {
    z0p_gpu_ctx* c = nullptr;
    int rc = z0p_gpu_ctx_create(device, &c);
    if (rc) {
      for (auto* x : p->ctxs) z0p_gpu_ctx_destroy(x);
      delete p;
      return rc;
    }
    p->ctxs.push_back(c);
  }
  for (auto* c : p->ctxs) p->threads.emplace_back(worker, p, c);
  *out = p;
  return Z0P_OK;
}

void z0p_gpu_pool_destroy(z0p_gpu_pool* p) {
  if (!p) return;
  {
    // Jobs still queued are cancelled; running ones finish first.
    std::lock_guard<std::mutex> lk(p->mu);
    p->stop = true;
    for (auto& item : p->queue) {
      item.job->status = Z0P_ERR_CANCELLED;
      p->done[item.ticket] = Z0P_ERR_CANCELLED;
    }
    p->queue.clear();
  }
  p->work_cv.notify_all();
  p->done_cv.notify_all();
  for (auto& t : p->threads) t.join();
  for (auto* c : p->ctxs) z0p_gpu_ctx_destroy(c);
  delete p;
}

int z0p_gpu_pool_submit(z0p_gpu_pool* p, z0p_job* job, uint64_t* ticket) {
  if (!p || !job || !ticket || !job->transcript) return Z0P_ERR_INVALID_ARGUMENT;
  size_t fp = 0;
  int rc = footprint(job, &fp);
  if (rc) return rc;
  if (fp > p->budget) {
    z0p::host::set_reason("job footprint exceeds the pool's HBM budget");
    return Z0P_ERR_ADMISSION;
  }
  {
    std::lock_guard<std::mutex> lk(p->mu);
    if (p->stop) return Z0P_ERR_CANCELLED;
    job->status = -1;
    job->submit_s = p->now();
    *ticket = p->next_ticket++;
    p->queue.push_back(Pending{job, *ticket, fp});
  }
  p->work_cv.notify_all();
  return Z0P_OK;
}

int z0p_gpu_pool_wait(z0p_gpu_pool* p, uint64_t ticket, int timeout_ms) {
  if (!p) return Z0P_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(p->mu);
  auto ready = [&] { return p->done.count(ticket) != 0; };
  if (timeout_ms < 0) {
    p->done_cv.wait(lk, ready);
  } else if (!p->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    return Z0P_ERR_DEVICE_TIMEOUT;
  }
  int rc = p->done[ticket];
  p->done.erase(ticket);
  return rc;
}

int z0p_gpu_pool_prove_all(z0p_gpu_pool* p, z0p_job* jobs, size_t n) {
  if (!p || (!jobs && n)) return Z0P_ERR_INVALID_ARGUMENT;
  std::vector<std::pair<size_t, size_t>> order;  // (footprint, index)
  for (size_t i = 0; i < n; i++) {
    size_t fp = 0;
    int rc = footprint(&jobs[i], &fp);
    if (rc) {
      jobs[i].status = rc;
      return rc;
    }
    order.push_back({fp, i});
  }
  std::stable_sort(order.begin(), order.end(),
                   [](const auto& a, const auto& b) { return a.first > b.first; });
  std::vector<uint64_t> tickets(n, 0);
  int first_err = Z0P_OK;
  for (auto& o : order) {
    int rc = z0p_gpu_pool_submit(p, &jobs[o.second], &tickets[o.second]);
    if (rc) {
      jobs[o.second].status = rc;
      if (!first_err) first_err = rc;
    }
  }
  for (size_t i = 0; i < n; i++) {
    if (!tickets[i]) continue;
    int rc = z0p_gpu_pool_wait(p, tickets[i], -1);
    if (rc && !first_err) first_err = rc;
  }
  return first_err;
}

double z0p_gpu_pool_clock(z0p_gpu_pool* p) { return p ? p->now() : 0.0; }

}  // extern "C"
