// pps_serve.cu -- a request server with continuous batching of swarms.
//
// The reference has no serving layer: each solve() owns the device for its
// duration.  This server admits optimization problems as they arrive and
// solves small swarms in the batched kernel (one CTA or cluster per swarm,
// all iterations in one launch, pps_batch.cu).  Large swarms (at least
// `single_min_n` particles, or `ode_single_min_n` for ODE fits) and MLP fits,
// whose loss runs on the tensor cores with one CTA per SM and tile
// (pps_mlp.cu), run instead as a swarm of their own on a launch slot with the
// multi-block step kernels of a plain solve (state carved from the same
// arena, iterations replayed as a CUDA graph, the result written to the
// request's mailbox by a last kernel), concurrently with the batched launches
// on the other slots.  Every other slot's stream has the device's highest
// priority and batched launches prefer those, so their persistent CTAs are
// placed ahead of the per-iteration blocks of the swarms run on their own:
//
//   submit()  validates the problem, stamps the arrival time and queues it.
//   worker    one host thread that, in a loop,
//               - retires finished requests: each swarm's CTAs write its
//                 result and then a done flag into mapped host memory, so a
//                 request completes when its own swarm does, not when its
//                 launch does; the worker records its time-to-solution and
//                 returns its arena block at once;
//               - admits queued requests while their swarm state fits in the
//                 device arena (HBM budget fixed at start) and a launch slot is
//                 free: the head of the queue fixes the pack's cluster size
//                 (CTAs per swarm) and queued requests of that size join it;
//               - packs them into one k_batch launch on the slot's stream
//                 (longest work first).
//             Up to `max_launches` launches are in flight on separate streams,
//             so requests that arrive while others run start at once on the
//             SMs the running ones leave free: their work overlaps on the GPU.
//   poll()/wait()  hand back (u, cost, idx, latency) and free the request.
//
// Every swarm's result equals its solve alone (pps_sync_run on the same
// problem and seed, bit for bit): a swarm's arithmetic and random stream do
// not depend on the launch, slot or CTA that computes it.  Nothing on the
// device waits for the host or for another CTA.
#include <algorithm>
#include <cmath>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pps_arena.h"
#include "pps_batch.h"

namespace pps {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  BatchSwarm desc{};
  std::vector<float> host;  // lb | ub | u0 | data
  // a request solved as a swarm of its own (MLP fit): its problem, run
  // parameters and, while it runs, the swarm
  bool single = false;
  pps_problem prob{};
  float params[8] = {};
  int64_t n = 0;
  uint64_t seed = 0;
  int32_t maxiters = 0;
  float w = 0, wdamp = 0, c1 = 0, c2 = 0;
  pps_swarm* sw = nullptr;
  size_t bytes = 0, offset = 0;
  Clock::time_point t_submit, t_done;
  int state = 0;  // 0 queued, 1 running, 2 done
  std::vector<float> u;
  float cost = 0.0f;
  int64_t idx = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;
  bool high = false;             // a high-priority stream (preferred by batched launches)
  cudaEvent_t done = nullptr;
  BatchSwarm* ddescs = nullptr;
  int* dorder = nullptr;
  BatchSwarm* hdescs = nullptr;  // pinned
  int* horder = nullptr;         // pinned
  float* mail = nullptr;         // pinned, mapped: per request dim + 2 floats
  float* mail_dev = nullptr;
  int* flags = nullptr;          // pinned, mapped: per request done flag
  int* flags_dev = nullptr;
  std::vector<Request*> reqs;
  int open = 0;                  // requests of this launch not retired yet
  bool busy = false;
};


}  // namespace pps

using namespace pps;

struct pps_server {
  pps_serve_config cfg{};
  int device = 0;
  void* arena_mem = nullptr;
  Arena arena;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, Request*> reqs;
  std::thread worker;
  bool stop = false;
  uint64_t next_ticket = 1;
  // stats
  uint64_t submitted = 0, completed = 0, launches = 0, packed = 0;
  std::vector<double> lat_ms;
  Clock::time_point t_first{}, t_last{};
  bool any = false;
  int worker_error = 0;
  char worker_msg[256] = "";
};

namespace {

constexpr int kMaxPack = 4096;

int launch_pack(pps_server* s, Slot& sl, std::vector<Request*>& pack, const LaunchGroup& key) {
  const int ns = (int)pack.size();
  LaunchGroup g = key;
  g.offset = 0;
  g.count = ns;
  g.maxdim = 1;
  const size_t mstride = (size_t)kBatchMaxDim + 2;
  for (int k = 0; k < ns; ++k) {
    Request* r = pack[k];
    BatchSwarm& d = r->desc;
    const int D = d.dim;
    PPS_CUDA(cudaMemcpyAsync(const_cast<float*>(d.lb), r->host.data(), sizeof(float) * D, cudaMemcpyHostToDevice,
                             sl.stream));
    PPS_CUDA(cudaMemcpyAsync(const_cast<float*>(d.ub), r->host.data() + D, sizeof(float) * D, cudaMemcpyHostToDevice,
                             sl.stream));
    PPS_CUDA(cudaMemcpyAsync(const_cast<float*>(d.u0), r->host.data() + 2 * D, sizeof(float) * D,
                             cudaMemcpyHostToDevice, sl.stream));
    if (d.ndata)
      PPS_CUDA(cudaMemcpyAsync(const_cast<float*>(d.data), r->host.data() + 3 * D, sizeof(float) * (size_t)d.ndata,
                               cudaMemcpyHostToDevice, sl.stream));
    d.mail = sl.mail_dev + (size_t)k * mstride;
    d.done = sl.flags_dev + k;
    sl.flags[k] = 0;
    sl.hdescs[k] = d;
    g.maxdim = std::max(g.maxdim, D);
    g.data_floats = std::max(g.data_floats, (int)d.ndata);
    g.maxn = std::max(g.maxn, d.n);
  }
  std::vector<int> order(ns);
  for (int k = 0; k < ns; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return batch_work_estimate(pack[a]->desc) > batch_work_estimate(pack[c]->desc);
  });
  memcpy(sl.horder, order.data(), sizeof(int) * ns);
  PPS_CUDA(cudaMemcpyAsync(sl.ddescs, sl.hdescs, sizeof(BatchSwarm) * ns, cudaMemcpyHostToDevice, sl.stream));
  PPS_CUDA(cudaMemcpyAsync(sl.dorder, sl.horder, sizeof(int) * ns, cudaMemcpyHostToDevice, sl.stream));
  const int rc = batch_launch_group(sl.stream, sl.ddescs, sl.dorder, g, s->cfg.ppt);
  if (rc) return rc;
  PPS_CUDA(cudaEventRecord(sl.done, sl.stream));
  sl.reqs = pack;
  sl.open = ns;
  sl.busy = true;
  for (Request* r : pack) r->state = 1;
  s->launches++;
  s->packed += (uint64_t)ns;
  return PPS_OK;
}

// a request solved as a swarm of its own on slot `sl`: attach it to its arena
// block, init, the iterations (graph replays) and the mailbox write
int launch_single(pps_server* s, Slot& sl, Request* r) {
  int rc = swarm_attach(&r->prob, r->n, r->seed, 0u, static_cast<char*>(s->arena_mem) + r->offset, sl.stream, &r->sw);
  if (rc) return rc;
  sl.flags[0] = 0;
  if ((rc = swarm_enqueue_init(r->sw)) || (rc = swarm_enqueue_run(r->sw, r->maxiters, r->w, r->wdamp, r->c1, r->c2)) ||
      (rc = launch_publish_result(r->sw, sl.mail_dev, sl.flags_dev))) {
    cudaStreamSynchronize(sl.stream);
    swarm_detach(r->sw);
    r->sw = nullptr;
    return rc;
  }
  PPS_CUDA(cudaEventRecord(sl.done, sl.stream));
  sl.reqs.assign(1, r);
  sl.open = 1;
  sl.busy = true;
  r->state = 1;
  s->launches++;
  s->packed += 1;
  return PPS_OK;
}

// retire the requests of `sl` whose swarms have finished; free the slot when
// its launch has ended and every request is retired
bool retire_ready(pps_server* s, Slot& sl) {
  bool any = false;
  const size_t mstride = (size_t)kBatchMaxDim + 2;
  for (size_t k = 0; k < sl.reqs.size(); ++k) {
    Request* r = sl.reqs[k];
    if (!r || r->state == 2) continue;
    if (reinterpret_cast<volatile int*>(sl.flags)[k] == 0) continue;
    std::atomic_thread_fence(std::memory_order_acquire);
    const auto now = Clock::now();
    const float* o = sl.mail + k * mstride;
    r->u.assign(o, o + r->desc.dim);
    r->cost = o[r->desc.dim];
    uint32_t bits;
    memcpy(&bits, &o[r->desc.dim + 1], 4);
    r->idx = (int64_t)bits;
    r->t_done = now;
    r->state = 2;
    if (r->sw) {  // its stream has passed the mailbox write: the graph is idle
      swarm_detach(r->sw);
      r->sw = nullptr;
    }
    s->arena.release(r->offset, r->bytes);
    s->completed++;
    s->lat_ms.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
    s->t_last = now;
    sl.reqs[k] = nullptr;
    sl.open--;
    any = true;
  }
  if (sl.busy && sl.open == 0 && cudaEventQuery(sl.done) == cudaSuccess) {
    sl.reqs.clear();
    sl.busy = false;
    any = true;
  }
  return any;
}

void worker_main(pps_server* s) {
  cudaSetDevice(s->device);
  const auto tick = std::chrono::microseconds((int64_t)s->cfg.tick_us);
  std::unique_lock<std::mutex> lock(s->mu);
  while (true) {
    bool progressed = false;
    for (Slot& sl : s->slots)
      if (sl.busy) progressed |= retire_ready(s, sl);
    if (progressed) s->cv_done.notify_all();
    if (s->stop && s->queue.empty()) {
      bool busy = false;
      for (Slot& sl : s->slots) busy |= sl.busy;
      if (!busy) break;
    }
    Slot *free_slot = nullptr, *free_high = nullptr, *free_low = nullptr;
    int inflight = 0;
    for (Slot& sl : s->slots) {
      if (sl.busy)
        ++inflight;
      else if (sl.high && !free_high)
        free_high = &sl;
      else if (!sl.high && !free_low)
        free_low = &sl;
    }
    // a swarm of its own prefers a normal-priority slot, a batched launch a
    // high-priority one; either takes the other kind when its own is busy
    const bool head_single = !s->queue.empty() && s->queue.front()->single;
    free_slot = head_single ? (free_low ? free_low : free_high) : (free_high ? free_high : free_low);
    if (free_slot && !s->queue.empty() && s->queue.front()->single) {
      Request* r = s->queue.front();
      size_t off;
      if (s->arena.alloc(r->bytes, &off)) {
        s->queue.pop_front();
        r->offset = off;
        const int rc = launch_single(s, *free_slot, r);
        if (rc) {
          s->worker_error = rc;
          snprintf(s->worker_msg, sizeof(s->worker_msg), "%s", pps_last_error());
          s->arena.release(r->offset, r->bytes);
          r->state = 2;
          r->cost = NAN;
          r->idx = -1;
          r->t_done = Clock::now();
          s->cv_done.notify_all();
        }
        continue;
      }
    } else if (free_slot && !s->queue.empty()) {
      const auto waited = Clock::now() - s->queue.front()->t_submit;
      if (inflight == 0 || waited >= tick || (int)s->queue.size() >= s->cfg.max_pack) {
        // the head of the queue fixes the launch shape (kernel, block and
        // cluster size); queued requests of the same shape join its pack in
        // arrival order
        const LaunchGroup key = batch_group_of(s->queue.front()->desc, s->cfg.threads, s->cfg.ppt);
        std::vector<Request*> pack;
        size_t scanned = 0;
        for (auto it = s->queue.begin(); it != s->queue.end() && (int)pack.size() < s->cfg.max_pack &&
                                         scanned < 4 * (size_t)s->cfg.max_pack;
             ++scanned) {
          Request* r = *it;
          if (r->single) {
            ++it;
            continue;
          }
          const LaunchGroup gr = batch_group_of(r->desc, s->cfg.threads, s->cfg.ppt);
          if (gr.kind != key.kind || gr.T != key.T || gr.C != key.C) {
            ++it;
            continue;
          }
          size_t off;
          if (!s->arena.alloc(r->bytes, &off)) break;  // memory-bound: wait for completions
          it = s->queue.erase(it);
          r->offset = off;
          batch_carve(r->desc, static_cast<char*>(s->arena_mem) + off);
          pack.push_back(r);
        }
        if (!pack.empty()) {
          const int rc = launch_pack(s, *free_slot, pack, key);
          if (rc) {
            s->worker_error = rc;
            snprintf(s->worker_msg, sizeof(s->worker_msg), "%s", pps_last_error());
            for (Request* r : pack) {
              s->arena.release(r->offset, r->bytes);
              r->state = 2;
              r->cost = NAN;
              r->idx = -1;
              r->t_done = Clock::now();
            }
            s->cv_done.notify_all();
          }
          continue;
        }
      }
    }
    // sleep until a submit or the next poll of the running swarms
    s->cv_work.wait_for(lock, std::chrono::microseconds(inflight ? 20 : 500));
  }
}

}  // namespace

extern "C" {

int pps_serve_start(const pps_serve_config* cfg_in, pps_server** out) {
  if (!out) return set_error(PPS_EINVAL, "out is NULL");
  *out = nullptr;
  pps_serve_config cfg = cfg_in ? *cfg_in : pps_serve_config{};
  if (cfg.memory_budget == 0) cfg.memory_budget = (uint64_t)8 << 30;
  if (cfg.max_launches <= 0) cfg.max_launches = 8;
  if (cfg.max_pack <= 0) cfg.max_pack = 512;
  if (cfg.threads == 0) cfg.threads = 256;
  if (cfg.ppt == 0) cfg.ppt = 1;
  if (cfg.tick_us < 0) cfg.tick_us = 0;
  if (cfg.single_min_n == 0) cfg.single_min_n = 2048;
  if (cfg.max_launches > 64 || cfg.max_pack > kMaxPack)
    return set_error(PPS_EINVAL, "max_launches <= 64 and max_pack <= %d", kMaxPack);
  if (!(cfg.threads == 128 || cfg.threads == 256 || cfg.threads == 512) ||
      !(cfg.ppt == 1 || cfg.ppt == 2 || cfg.ppt == 4))
    return set_error(PPS_EINVAL, "threads in {128, 256, 512}, ppt in {1, 2, 4}");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return set_error(PPS_ENODEV, "no CUDA device");
  pps_server* s = new (std::nothrow) pps_server();
  if (!s) return set_error(PPS_ENOMEM, "host allocation failed");
  s->cfg = cfg;
  cudaGetDevice(&s->device);
  cudaError_t e = cudaMalloc(&s->arena_mem, cfg.memory_budget);
  if (e != cudaSuccess) {
    delete s;
    return cuda_error(e, "cudaMalloc(serving arena)");
  }
  s->arena.reset(cfg.memory_budget);
  s->slots.resize(cfg.max_launches);
  const size_t mail_floats = (size_t)cfg.max_pack * (kBatchMaxDim + 2);
  // every other slot's stream has the device's highest priority: batched
  // launches take those, so their persistent CTAs are placed ahead of the
  // blocks of swarms run on their own, which relaunch every iteration
  int prio_low = 0, prio_high = 0;
  if ((e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high)) != cudaSuccess) {
    const int rc = cuda_error(e, "cudaDeviceGetStreamPriorityRange");
    pps_serve_stop(s);
    return rc;
  }
  for (size_t k = 0; k < s->slots.size(); ++k) s->slots[k].high = (k % 2) == 0;
  for (Slot& sl : s->slots) {
    if ((e = cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, sl.high ? prio_high : prio_low)) !=
            cudaSuccess ||
        (e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaMalloc(&sl.ddescs, sizeof(BatchSwarm) * cfg.max_pack)) != cudaSuccess ||
        (e = cudaMalloc(&sl.dorder, sizeof(int) * cfg.max_pack)) != cudaSuccess ||
        (e = cudaMallocHost(&sl.hdescs, sizeof(BatchSwarm) * cfg.max_pack)) != cudaSuccess ||
        (e = cudaMallocHost(&sl.horder, sizeof(int) * cfg.max_pack)) != cudaSuccess ||
        (e = cudaHostAlloc(&sl.mail, sizeof(float) * mail_floats, cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaHostAlloc(&sl.flags, sizeof(int) * cfg.max_pack, cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer(&sl.mail_dev, sl.mail, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer(&sl.flags_dev, sl.flags, 0)) != cudaSuccess) {
      const int rc = cuda_error(e, "serving slot allocation");
      pps_serve_stop(s);
      return rc;
    }
  }
  s->worker = std::thread(worker_main, s);
  *out = s;
  return PPS_OK;
}

int pps_serve_submit(pps_server* s, const pps_problem* prob, int64_t n, uint64_t seed, int32_t maxiters, float w,
                     float wdamp, float c1, float c2, uint64_t* ticket) {
  if (!s || !ticket) return set_error(PPS_EINVAL, "NULL argument");
  Request* r = new (std::nothrow) Request();
  if (!r) return set_error(PPS_ENOMEM, "host allocation failed");
  // MLP fits (the tensor-core kernel wants whole SMs), constrained problems,
  // user objectives, Tsit5 ODE fits and large swarms run as a swarm of their
  // own with the multi-block step kernels; the rest are packed into batched
  // launches
  const bool tsit5 = prob && is_ode(prob->objective) && prob->nparams > 6 && prob->params && prob->params[6] != 0.0f;
  const int32_t min_n = prob && is_ode(prob->objective) && s->cfg.ode_single_min_n != 0 ? s->cfg.ode_single_min_n
                                                                                        : s->cfg.single_min_n;
  const bool single = prob && (prob->objective == kMlp || prob->ncons > 0 || is_user(prob->objective) || tsit5 ||
                               (min_n > 0 && n >= min_n));
  if (single) {
    int rc = swarm_check(prob, n);
    if (!rc && prob->dim > kBatchMaxDim)
      rc = set_error(PPS_EINVAL, "served problems have at most %d dims (got %d)", kBatchMaxDim, prob->dim);
    if (!rc && maxiters < 0) rc = set_error(PPS_EINVAL, "maxiters must be >= 0");
    if (!rc && !(std::isfinite(w) && std::isfinite(wdamp) && std::isfinite(c1) && std::isfinite(c2)))
      rc = set_error(PPS_EINVAL, "coefficients must be finite");
    if (rc) {
      delete r;
      return rc;
    }
    const int D = prob->dim;
    r->single = true;
    r->host.resize((size_t)3 * D + (size_t)prob->ndata);
    for (int d = 0; d < D; ++d) {
      r->host[d] = prob->lb ? prob->lb[d] : -INFINITY;
      r->host[D + d] = prob->ub ? prob->ub[d] : INFINITY;
      r->host[2 * D + d] = prob->u0 ? prob->u0[d] : 0.0f;
    }
    if (prob->data && prob->ndata > 0) memcpy(r->host.data() + 3 * D, prob->data, sizeof(float) * (size_t)prob->ndata);
    for (int k = 0; k < prob->nparams; ++k) r->params[k] = prob->params[k];
    r->prob = *prob;
    r->prob.lb = r->host.data();
    r->prob.ub = r->host.data() + D;
    r->prob.u0 = r->host.data() + 2 * D;
    r->prob.data = (prob->data && prob->ndata > 0) ? r->host.data() + 3 * D : nullptr;
    r->prob.ndata = (prob->data && prob->ndata > 0) ? prob->ndata : 0;
    r->prob.params = r->params;
    r->n = n;
    r->seed = seed;
    r->maxiters = maxiters;
    r->w = w;
    r->wdamp = wdamp;
    r->c1 = c1;
    r->c2 = c2;
    r->desc.dim = D;
    r->bytes = (swarm_device_bytes(prob, n) + 255) / 256 * 256;
  } else {
    const int rc = batch_describe(prob, n, seed, maxiters, w, wdamp, c1, c2, &r->desc, &r->host);
    if (rc) {
      delete r;
      return rc;
    }
    r->bytes = batch_swarm_bytes(r->desc.dim, r->desc.ld, r->desc.ndata);
  }
  if (r->bytes > s->cfg.memory_budget) {
    const size_t need = r->bytes;
    delete r;
    return set_error(PPS_ENOMEM, "request needs %zu bytes, more than the serving arena (%llu)", need,
                     (unsigned long long)s->cfg.memory_budget);
  }
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) {
      delete r;
      return set_error(PPS_EINVAL, "server is stopping");
    }
    r->ticket = s->next_ticket++;
    s->reqs[r->ticket] = r;
    s->queue.push_back(r);
    s->submitted++;
    if (!s->any) {
      s->t_first = r->t_submit;
      s->any = true;
    }
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  return PPS_OK;
}

static int take_result(pps_server* s, Request* r, float* u, float* cost, int64_t* idx, double* latency_ms) {
  if (u) memcpy(u, r->u.data(), sizeof(float) * r->u.size());
  if (cost) *cost = r->cost;
  if (idx) *idx = r->idx;
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  const bool failed = r->idx < 0;
  s->reqs.erase(r->ticket);
  delete r;
  if (failed) return set_error(s->worker_error ? s->worker_error : PPS_ECUDA, "launch failed: %s", s->worker_msg);
  return PPS_OK;
}

int pps_serve_poll(pps_server* s, uint64_t ticket, float* u, float* cost, int64_t* idx, double* latency_ms) {
  if (!s) return set_error(PPS_EINVAL, "server is NULL");
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return set_error(PPS_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
  if (it->second->state != 2) return PPS_EBUSY;
  return take_result(s, it->second, u, cost, idx, latency_ms);
}

int pps_serve_wait(pps_server* s, uint64_t ticket, float* u, float* cost, int64_t* idx, double* latency_ms,
                   double timeout_s) {
  if (!s) return set_error(PPS_EINVAL, "server is NULL");
  if (std::isnan(timeout_s)) return set_error(PPS_EINVAL, "timeout_s is NaN");
  // negative: no wait; at most about a year, so the deadline stays representable
  const double limit_s = timeout_s < 0.0 ? 0.0 : std::min(timeout_s, 3.0e7);
  std::unique_lock<std::mutex> lock(s->mu);
  const auto deadline =
      Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(limit_s));
  while (true) {
    // looked up again after every wake-up: another caller may have taken the
    // result (and freed the request) meanwhile
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(PPS_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
    if (it->second->state == 2) return take_result(s, it->second, u, cost, idx, latency_ms);
    if (s->cv_done.wait_until(lock, deadline) == std::cv_status::timeout) {
      it = s->reqs.find(ticket);
      if (it != s->reqs.end() && it->second->state == 2) return take_result(s, it->second, u, cost, idx, latency_ms);
      if (it == s->reqs.end()) return set_error(PPS_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
      return set_error(PPS_ETIMEOUT, "request %llu not done within %.3f s", (unsigned long long)ticket, limit_s);
    }
  }
}

int pps_serve_stats_get(pps_server* s, pps_serve_stats* st) {
  if (!s || !st) return set_error(PPS_EINVAL, "NULL argument");
  std::lock_guard<std::mutex> lock(s->mu);
  memset(st, 0, sizeof(*st));
  st->submitted = s->submitted;
  st->completed = s->completed;
  st->launches = s->launches;
  st->mean_pack = s->launches ? (double)s->packed / (double)s->launches : 0.0;
  st->arena_bytes = s->cfg.memory_budget;
  st->arena_peak_bytes = s->arena.peak();
  st->queued = (int32_t)s->queue.size();
  int running = 0;
  for (Slot& sl : s->slots) running += sl.open;
  st->running = running;
  if (!s->lat_ms.empty()) {
    std::vector<double> v = s->lat_ms;
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) {
      const size_t k = (size_t)std::min<double>((double)v.size() - 1, std::floor(q * (double)(v.size() - 1) + 0.5));
      return v[k];
    };
    st->p50_ms = pct(0.50);
    st->p99_ms = pct(0.99);
    st->max_ms = v.back();
    double sum = 0;
    for (double x : v) sum += x;
    st->mean_ms = sum / (double)v.size();
    const double span = std::chrono::duration<double>(s->t_last - s->t_first).count();
    st->solves_per_s = span > 0 ? (double)s->completed / span : 0.0;
  }
  return PPS_OK;
}

int pps_serve_stop(pps_server* s) {
  if (!s) return PPS_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (Slot& sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.ddescs) cudaFree(sl.ddescs);
    if (sl.dorder) cudaFree(sl.dorder);
    if (sl.hdescs) cudaFreeHost(sl.hdescs);
    if (sl.horder) cudaFreeHost(sl.horder);
    if (sl.mail) cudaFreeHost(sl.mail);
    if (sl.flags) cudaFreeHost(sl.flags);
  }
  for (auto& kv : s->reqs) {
    if (kv.second->sw) swarm_detach(kv.second->sw);
    delete kv.second;
  }
  if (s->arena_mem) cudaFree(s->arena_mem);
  delete s;
  return PPS_OK;
}

}  // extern "C"
