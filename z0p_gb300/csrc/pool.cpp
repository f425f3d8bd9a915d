// Batched and served proving: a pool of prover contexts fed by a FIFO queue
// with HBM-footprint admission (include/z0p_gpu.h, "batching / serving").
//
// Each worker thread owns one context (its own CUDA stream and workspace),
// so independent proofs overlap on the GPU: one proof's kernels fill the
// SMs while another waits on its Fiat-Shamir round trip. A worker that
// takes the queue head also takes the queued jobs of the same shape behind
// it that fit the budget, up to a group limit, and proves them as one
// lockstep group (one launch sequence and one set of round trips): requests
// that arrive while others run are batched as they come. Admission keeps the
// sum of running jobs' device footprints within the budget; the head is
// always served first, so a large job is never starved by smaller ones.
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
#include "kernels.h"

namespace {

constexpr size_t kKeepBytes = 512ull << 20;  // workspace an idle worker may keep
// A group holds at most kGroupMax proofs and about kGroupRows LDE rows in all:
// small proofs group widely (their kernels and round trips are mostly fixed
// cost), a proof whose LDE alone fills the GPU stays alone.
constexpr uint32_t kGroupMax = 16;
constexpr uint64_t kGroupRows = 1ull << 22;

struct Pending {
  z0p_job* job;
  uint64_t ticket;
  size_t footprint;
};

bool same_shape(const z0p_job* a, const z0p_job* b) {
  if (a->kind != b->kind) return false;
  if (a->kind == Z0P_JOB_AIR)
    return a->air.n_steps == b->air.n_steps && a->air.blowup == b->air.blowup &&
           a->air.num_queries == b->air.num_queries && a->air.final_size == b->air.final_size &&
           a->air.grinding_bits == b->air.grinding_bits && a->air.cap_height == b->air.cap_height;
  return a->range.n_rows == b->range.n_rows && a->range.n_bits == b->range.n_bits &&
         a->range.blowup == b->range.blowup && a->range.num_queries == b->range.num_queries &&
         a->range.final_size == b->range.final_size &&
         a->range.grinding_bits == b->range.grinding_bits &&
         a->range.cap_height == b->range.cap_height;
}

// `slots`: the worker's reserved group size (constant slots).
uint32_t group_limit(const z0p_job* j, uint32_t slots) {
  uint64_t rows = j->kind == Z0P_JOB_AIR ? j->air.n_steps * j->air.blowup
                                         : j->range.n_rows * j->range.blowup * (j->range.n_bits + 1);
  uint64_t g = rows ? kGroupRows / rows : 1;
  const uint32_t most = kGroupMax < slots ? kGroupMax : slots;
  return g < 1 ? 1u : (g > most ? most : (uint32_t)g);
}

}  // namespace

struct z0p_gpu_pool {
  int device = 0;
  std::vector<z0p_gpu_ctx*> ctxs;
  std::vector<uint32_t> slots;  // per worker: the group size its context reserved
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

// Proves one group of same-shape jobs on the worker's context.
int prove_group(z0p_gpu_ctx* ctx, const std::vector<Pending>& group) {
  const size_t n = group.size();
  std::vector<z0p_transcript_state*> ts(n);
  std::vector<uint8_t*> outs(n);
  std::vector<size_t> caps(n), lens(n, 0);
  for (size_t i = 0; i < n; i++) {
    ts[i] = group[i].job->transcript;
    outs[i] = group[i].job->out;
    caps[i] = group[i].job->cap;
  }
  int rc;
  if (group[0].job->kind == Z0P_JOB_AIR) {
    std::vector<z0p_air_params> ps(n);
    for (size_t i = 0; i < n; i++) ps[i] = group[i].job->air;
    rc = z0p_gpu_air_prove_group(ctx, n, ps.data(), ts.data(), outs.data(), caps.data(), lens.data());
  } else {
    std::vector<z0p_range_params> ps(n);
    for (size_t i = 0; i < n; i++) ps[i] = group[i].job->range;
    rc = z0p_gpu_range_prove_group(ctx, n, ps.data(), ts.data(), outs.data(), caps.data(),
                                   lens.data());
  }
  for (size_t i = 0; i < n; i++) group[i].job->len = lens[i];
  return rc;
}

void worker(z0p_gpu_pool* p, z0p_gpu_ctx* ctx, uint32_t slots) {
  cudaSetDevice(p->device);
  for (;;) {
    std::vector<Pending> group;
    size_t group_fp = 0;
    {
      std::unique_lock<std::mutex> lk(p->mu);
      // FIFO head first, admitted when it fits next to the running jobs.
      p->work_cv.wait(lk, [&] {
        return p->stop ||
               (!p->queue.empty() && p->inflight + p->queue.front().footprint <= p->budget);
      });
      if (p->stop) return;
      group.push_back(p->queue.front());
      p->queue.pop_front();
      group_fp = group[0].footprint;
      // Then the queued jobs of the same shape, while they fit.
      const uint32_t limit = group_limit(group[0].job, slots);
      for (auto it = p->queue.begin(); it != p->queue.end() && group.size() < limit;) {
        if (same_shape(it->job, group[0].job) &&
            p->inflight + group_fp + it->footprint <= p->budget) {
          group_fp += it->footprint;
          group.push_back(*it);
          it = p->queue.erase(it);
        } else {
          ++it;
        }
      }
      p->inflight += group_fp;
      const double t = p->now();
      for (auto& g : group) g.job->start_s = t;
    }
    // The next head may fit too.
    p->work_cv.notify_all();
    int rc = prove_group(ctx, group);
    // A context that just held a large job gives its workspace back to the
    // device pool, so memory held by idle workers stays small next to the
    // admission budget.
    if (z0p_gpu_ctx_device_bytes(ctx) > kKeepBytes) z0p_gpu_ctx_trim(ctx);
    {
      std::lock_guard<std::mutex> lk(p->mu);
      const double t = p->now();
      for (auto& g : group) {
        g.job->status = rc;
        g.job->end_s = t;
        p->done[g.ticket] = rc;
      }
      p->inflight -= group_fp;
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
    // Side by side, a worker's proofs overlap the others' latency-bound
    // stages; launches waiting at gates would only hold SM slots.
    if (workers > 1) z0p_gpu_ctx_set_gates(c, 0);
    p->ctxs.push_back(c);
  }
  // Each worker reserves constant slots for its groups: an equal share of
  // the process's slots (a few kept for other contexts), at most kGroupMax,
  // or less when other contexts already hold slots.
  const int spare = z0p::kConstSlots - 8 - workers;
  uint32_t share = spare > 0 ? 1u + (uint32_t)(spare / workers) : 1u;
  if (share > kGroupMax) share = kGroupMax;
  for (auto* c : p->ctxs) {
    uint32_t g = share;
    while (g > 1 && z0p_gpu_ctx_reserve_group(c, g) != Z0P_OK) g--;
    p->slots.push_back(g);
  }
  for (size_t i = 0; i < p->ctxs.size(); i++)
    p->threads.emplace_back(worker, p, p->ctxs[i], p->slots[i]);
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
