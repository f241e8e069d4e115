// serve.cu - continuous batching of join requests (host code).
//
// Lanes: each owns a CUDA stream, an ej_handle (whose scratch arena persists
// across batches) and pinned/device count buffers.  A scheduler thread waits
// for queued requests and a free lane, admits requests in arrival order while
// the batch's device footprint stays within the lane budget (a request larger
// than the budget alone still runs, alone), launches the batch asynchronously
// and appends a host callback; the callback (a CUDA runtime thread, no CUDA
// calls) stamps completion times, publishes the completions and frees the
// lane.  So requests that arrive while others are on the GPU wait only for
// the next free lane, and the batches of different lanes overlap on the device.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "ej_internal.h"

extern "C" uint64_t ej_now_ns(void) {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

namespace {

struct Request {
  ej_join_desc join;
  uint64_t tag;
  uint64_t arrival_ns;
};

struct Lane;

struct Server {
  ej_server_config cfg{};
  std::vector<Lane*> lanes;
  std::mutex mu;
  std::condition_variable cv_sched;   // queue or lane state changed
  std::condition_variable cv_done;    // completions published
  std::deque<Request> queue;
  std::deque<ej_completion> done;
  uint64_t submitted = 0, completed = 0;
  bool stop = false;
  ej_status fatal = EJ_OK;
  std::thread sched;
};

struct Lane {
  Server* srv = nullptr;
  ej_handle* h = nullptr;
  cudaStream_t stream = nullptr;
  unsigned long long* d_counts = nullptr;
  unsigned long long* h_counts = nullptr;
  // EJ_SERVE_CHECKSUM: the batch's requests and their outputs' checksums
  ej_join_desc* d_desc = nullptr;
  ej_join_desc* h_desc = nullptr;
  unsigned long long* d_sums = nullptr;
  unsigned long long* h_sums = nullptr;
  uint32_t cap = 0;
  bool busy = false;
  ej_status launch_status = EJ_OK;
  uint64_t launch_ns = 0;
  std::vector<Request> batch;
};

// device scratch a request adds to a batch (see batch.cu / hash_join.cu layouts)
uint64_t footprint(const ej_join_desc& j, int mode) {
  const uint64_t per_r = mode == EJ_SERVE_BATCHED ? 34 : 44;
  return per_r * j.nR + 9 * j.nS + (1u << 20);
}

void CUDART_CB lane_done(void* arg) {
  Lane* L = static_cast<Lane*>(arg);
  Server* S = L->srv;
  const uint64_t now = ej_now_ns();
  {
    std::lock_guard<std::mutex> lock(S->mu);
    for (size_t i = 0; i < L->batch.size(); i++) {
      const Request& r = L->batch[i];
      ej_completion c;
      c.tag = r.tag;
      c.count = L->h_counts[i];
      c.status = L->launch_status != EJ_OK ? L->launch_status
                 : (c.count > r.join.out_cap ? EJ_ERR_CAPACITY : EJ_OK);
      c.batch_joins = (uint32_t)L->batch.size();
      c.arrival_ns = r.arrival_ns;
      c.launch_ns = L->launch_ns;
      c.done_ns = now;
      c.checksum = (S->cfg.flags & EJ_SERVE_CHECKSUM) ? L->h_sums[i] : 0;
      S->done.push_back(c);
    }
    S->completed += L->batch.size();
    L->batch.clear();
    L->busy = false;
  }
  S->cv_sched.notify_all();
  S->cv_done.notify_all();
}

ej_status lane_launch(Lane* L, int mode) {
  ej_handle* h = L->h;
  const uint32_t n = (uint32_t)L->batch.size();
  ej_status st = EJ_OK;
  if (mode == EJ_SERVE_BATCHED) {
    std::vector<ej_join_desc> d(n);
    for (uint32_t i = 0; i < n; i++) d[i] = L->batch[i].join;
    st = ej_batch_hash_join_async(h, d.data(), n, reinterpret_cast<uint64_t*>(L->d_counts));
  } else {
    for (uint32_t i = 0; i < n && st == EJ_OK; i++) {
      const ej_join_desc& j = L->batch[i].join;
      st = ej_hash_join_async(h, j.R, j.nR, j.S, j.nS, j.out, j.out_cap, reinterpret_cast<uint64_t*>(L->d_counts + i));
    }
  }
  if (st == EJ_OK && (L->srv->cfg.flags & EJ_SERVE_CHECKSUM)) {
    // the lane is busy until this batch completes, so h_desc is not rewritten
    // before its copy runs
    for (uint32_t i = 0; i < n; i++) L->h_desc[i] = L->batch[i].join;
    if (cudaMemcpyAsync(L->d_desc, L->h_desc, n * sizeof(ej_join_desc), cudaMemcpyHostToDevice, L->stream) !=
        cudaSuccess)
      st = EJ_ERR_CUDA;
    if (st == EJ_OK) st = ej_checksum_outputs_async(h, L->d_desc, L->d_counts, n, L->d_sums);
    if (st == EJ_OK && cudaMemcpyAsync(L->h_sums, L->d_sums, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                       L->stream) != cudaSuccess)
      st = EJ_ERR_CUDA;
  }
  if (st == EJ_OK && cudaMemcpyAsync(L->h_counts, L->d_counts, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                     L->stream) != cudaSuccess)
    st = EJ_ERR_CUDA;
  L->launch_status = st;
  if (st != EJ_OK) {
    // nothing (more) runs for this batch: report it failed without waiting on the device
    for (uint32_t i = 0; i < n; i++) L->h_counts[i] = 0;
    lane_done(L);
    return st;
  }
  if (cudaLaunchHostFunc(L->stream, lane_done, L) != cudaSuccess) {
    cudaGetLastError();
    L->launch_status = EJ_ERR_CUDA;
    cudaStreamSynchronize(L->stream);
    lane_done(L);
    return EJ_ERR_CUDA;
  }
  return EJ_OK;
}

void scheduler(Server* S) {
  cudaSetDevice(S->cfg.device);
  const uint32_t max_joins = S->cfg.mode == EJ_SERVE_PER_JOIN ? 1u : S->cfg.max_batch_joins;
  for (;;) {
    Lane* L = nullptr;
    {
      std::unique_lock<std::mutex> lock(S->mu);
      for (;;) {
        if (S->stop && S->queue.empty()) return;
        if (!S->queue.empty()) {
          for (Lane* c : S->lanes)
            if (!c->busy) {
              L = c;
              break;
            }
          if (L) break;
        }
        S->cv_sched.wait(lock);
      }
      // admit queued requests in arrival order within the lane's budget
      uint64_t bytes = 0;
      while (!S->queue.empty() && L->batch.size() < max_joins) {
        const uint64_t f = footprint(S->queue.front().join, S->cfg.mode);
        if (!L->batch.empty() && bytes + f > S->cfg.lane_bytes) break;
        bytes += f;
        L->batch.push_back(S->queue.front());
        S->queue.pop_front();
      }
      L->busy = true;
    }
    L->launch_ns = ej_now_ns();
    lane_launch(L, S->cfg.mode);
  }
}

void server_free(Server* S) {
  for (Lane* L : S->lanes) {
    if (L->stream) cudaStreamSynchronize(L->stream);
    if (L->h) ej_destroy(L->h);
    if (L->stream) cudaStreamDestroy(L->stream);
    cudaFree(L->d_counts);
    cudaFreeHost(L->h_counts);
    cudaFree(L->d_desc);
    cudaFreeHost(L->h_desc);
    cudaFree(L->d_sums);
    cudaFreeHost(L->h_sums);
    delete L;
  }
  delete S;
}

}  // namespace

struct ej_server {
  Server* s;
};

extern "C" ej_status ej_server_create(const ej_server_config* cfg, ej_server** out) {
  if (!cfg || !out) return EJ_ERR_INVALID;
  *out = nullptr;
  Server* S = new Server();
  S->cfg = *cfg;
  if (S->cfg.lanes == 0) S->cfg.lanes = 2;
  if (S->cfg.max_batch_joins == 0) S->cfg.max_batch_joins = 1024;
  if (S->cfg.lane_bytes == 0) S->cfg.lane_bytes = 16ull << 30;
  if (S->cfg.mode != EJ_SERVE_BATCHED && S->cfg.mode != EJ_SERVE_PER_JOIN) {
    delete S;
    return EJ_ERR_INVALID;
  }
  const uint32_t per_lane = S->cfg.mode == EJ_SERVE_PER_JOIN ? 1u : S->cfg.max_batch_joins;
  for (uint32_t i = 0; i < S->cfg.lanes; i++) {
    Lane* L = new Lane();
    L->srv = S;
    S->lanes.push_back(L);
    ej_status st = ej_create(cfg->device, &L->h);
    if (st != EJ_OK) {
      server_free(S);
      return st;
    }
    if (cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking) != cudaSuccess ||
        ej_dev_alloc(&L->d_counts, per_lane * sizeof(unsigned long long)) != cudaSuccess ||
        ej_host_alloc(&L->h_counts, per_lane * sizeof(unsigned long long)) != cudaSuccess ||
        ((S->cfg.flags & EJ_SERVE_CHECKSUM) &&
         (ej_dev_alloc(&L->d_desc, per_lane * sizeof(ej_join_desc)) != cudaSuccess ||
          ej_host_alloc(&L->h_desc, per_lane * sizeof(ej_join_desc)) != cudaSuccess ||
          ej_dev_alloc(&L->d_sums, per_lane * sizeof(unsigned long long)) != cudaSuccess ||
          ej_host_alloc(&L->h_sums, per_lane * sizeof(unsigned long long)) != cudaSuccess))) {
      cudaGetLastError();
      server_free(S);
      return EJ_ERR_NOMEM;
    }
    L->cap = per_lane;
    ej_set_stream(L->h, L->stream);
  }
  S->sched = std::thread(scheduler, S);
  ej_server* srv = new ej_server();
  srv->s = S;
  *out = srv;
  return EJ_OK;
}

extern "C" ej_status ej_server_submit(ej_server* srv, const ej_join_desc* join, uint64_t tag, uint64_t arrival_ns) {
  if (!srv || !join) return EJ_ERR_INVALID;
  if ((join->nR && !join->R) || (join->nS && !join->S) || (join->out_cap && !join->out)) return EJ_ERR_INVALID;
  Server* S = srv->s;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    if (S->stop) return EJ_ERR_BUSY;
    if (S->cfg.max_queued && S->queue.size() >= S->cfg.max_queued) return EJ_ERR_BUSY;  // admission refused
    S->queue.push_back({*join, tag, arrival_ns ? arrival_ns : ej_now_ns()});
    S->submitted++;
  }
  S->cv_sched.notify_all();
  return EJ_OK;
}

extern "C" ej_status ej_server_poll(ej_server* srv, ej_completion* out, uint32_t max, uint32_t* n, uint32_t wait_us) {
  if (!srv || !n || (max && !out)) return EJ_ERR_INVALID;
  Server* S = srv->s;
  std::unique_lock<std::mutex> lock(S->mu);
  if (S->done.empty() && wait_us)
    S->cv_done.wait_for(lock, std::chrono::microseconds(wait_us), [S] { return !S->done.empty(); });
  uint32_t k = 0;
  while (k < max && !S->done.empty()) {
    out[k++] = S->done.front();
    S->done.pop_front();
  }
  *n = k;
  return EJ_OK;
}

extern "C" ej_status ej_server_drain(ej_server* srv) {
  if (!srv) return EJ_ERR_INVALID;
  Server* S = srv->s;
  std::unique_lock<std::mutex> lock(S->mu);
  S->cv_done.wait(lock, [S] { return S->completed == S->submitted; });
  return EJ_OK;
}

extern "C" ej_status ej_server_destroy(ej_server* srv) {
  if (!srv) return EJ_ERR_INVALID;
  Server* S = srv->s;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
  }
  S->cv_sched.notify_all();
  if (S->sched.joinable()) S->sched.join();
  ej_server_drain(srv);
  server_free(S);
  delete srv;
  return EJ_OK;
}
