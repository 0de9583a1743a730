// Serving loop: continuous batching of search requests over resident
// collections (IVF-PQ, Flat, SQ8) on one GPU.
//
// Requests (a collection, nq query rows, k) are queued on submit; their
// rows are copied so the caller's buffer is free at once. A scheduler thread
// forms device batches: the oldest queued request picks the (collection, k)
// and every queued request with the same pair joins it in arrival order, up
// to a query limit. A batch is admitted when a lane is idle and its device
// memory estimate fits the HBM budget next to the batches in flight; lanes
// are worker threads, each with its own CUDA stream, pinned staging buffers
// and device buffers, so admitted batches overlap on the device while new
// requests keep arriving. Results are copied back through the lane's pinned
// buffer and scattered to the requests' output buffers; each request
// records its latency from submit to completion. A request with more rows
// than a batch may hold is split into parts of at most that many rows,
// queued together; it completes when its last part does.
//
// Each batch's device interval (events recorded on its lane's stream before
// the input copy and after the result copy) is kept, so the peak number of
// batches that were on the device at the same instant can be read back
// (mv_server_device_overlap).
//
// Every search path is deterministic per query (the selections do not
// depend on the other queries of a batch), so a request gets the same bits
// alone and in any mix.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mv_internal.h"

namespace {

using clk = std::chrono::steady_clock;

struct Coll {
  int kind;  // 0 IVF-PQ, 1 Flat, 2 SQ8
  void* handle;
  int d;
  mv_search_params params;
  int rerank_factor;
  size_t ws_per_query;  // device workspace estimate
  size_t ws_fixed;
};

struct Req {
  int64_t id;
  int coll;
  int k;
  int64_t nq;
  std::vector<float> x;
  float* out_d;
  int64_t* out_l;
  clk::time_point t_submit, t_done;
  int32_t status = 0;
  bool done = false;
  // A split request: the parent is not queued; its parts point at it and
  // it completes when parts_left reaches zero.
  Req* parent = nullptr;
  int parts_left = 0;
};

struct Batch {
  int coll = 0, k = 0;
  int64_t nq = 0;
  size_t bytes = 0;
  std::vector<Req*> reqs;
};

struct Lane {
  std::thread th;
  cudaStream_t s = nullptr;
  float* h_x = nullptr;  // pinned staging
  float* h_d = nullptr;
  int64_t* h_l = nullptr;
  size_t cap_x = 0, cap_d = 0, cap_l = 0;  // elements
  mv::DevBuf d_x, d_d, d_l;
  cudaEvent_t ev_a = nullptr, ev_b = nullptr;  // the batch's device interval
  std::unique_ptr<Batch> job;
  bool busy = false;
};

void grow_pinned(void** p, size_t& cap, size_t need, size_t elem) {
  if (need <= cap) return;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  const size_t n = std::max(need, cap * 2);
  MV_CHECK_CUDA(cudaHostAlloc(p, n * elem, cudaHostAllocDefault));
  cap = n;
}

}  // namespace

struct mv_server {
  mv_ctx* ctx;
  int64_t budget;
  int64_t max_batch;
  std::vector<Coll> colls;
  std::vector<std::unique_ptr<Lane>> lanes;
  std::deque<Req*> queue;
  std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
  std::vector<std::unique_ptr<Req>> parts;  // parts of split requests in flight
  cudaEvent_t ev_origin = nullptr;          // time base of the device intervals
  std::vector<std::pair<float, float>> intervals;  // device intervals of recent batches (ms)
  std::mutex mu;
  std::condition_variable cv_sched, cv_lane, cv_done;
  std::thread sched;
  bool stop = false;
  int64_t next_id = 1;
  int64_t in_flight_bytes = 0, peak_bytes = 0;
  int64_t batches = 0, batched_queries = 0, completed = 0;

  void lane_loop(Lane* ln);
  void sched_loop();
  void finish(Req* r, int32_t st, clk::time_point now);
  size_t estimate(const Coll& c, int64_t nq, int k) const {
    return (size_t)nq * (c.d * 4 + (size_t)k * 12) + c.ws_fixed + (size_t)nq * c.ws_per_query;
  }
};

void mv_server::sched_loop() {
  std::unique_lock<std::mutex> lk(mu);
  while (!stop) {
    bool admitted = false;
    if (!queue.empty()) {
      Lane* idle = nullptr;
      for (auto& l : lanes)
        if (!l->busy) {
          idle = l.get();
          break;
        }
      if (idle) {
        auto b = std::make_unique<Batch>();
        b->coll = queue.front()->coll;
        b->k = queue.front()->k;
        for (auto it = queue.begin(); it != queue.end();) {
          Req* r = *it;
          if (r->coll == b->coll && r->k == b->k && (b->nq == 0 || b->nq + r->nq <= max_batch)) {
            b->nq += r->nq;
            b->reqs.push_back(r);
            it = queue.erase(it);
          } else {
            ++it;
          }
        }
        b->bytes = colls[b->coll].kind >= 0 ? estimate(colls[b->coll], b->nq, b->k) : 0;
        const bool any_busy = in_flight_bytes > 0;
        if (any_busy && in_flight_bytes + (int64_t)b->bytes > budget) {
          // not admitted yet: back to the front of the queue, in order
          for (auto it = b->reqs.rbegin(); it != b->reqs.rend(); ++it) queue.push_front(*it);
        } else {
          in_flight_bytes += (int64_t)b->bytes;
          peak_bytes = std::max(peak_bytes, in_flight_bytes);
          ++batches;
          batched_queries += b->nq;
          idle->job = std::move(b);
          idle->busy = true;
          admitted = true;
          cv_lane.notify_all();
        }
      }
    }
    if (!admitted) cv_sched.wait(lk);
  }
}

void mv_server::lane_loop(Lane* ln) {
  mv_ctx* c = ctx;
  cudaSetDevice(c->device);
  while (true) {
    std::unique_ptr<Batch> b;
    Coll co;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_lane.wait(lk, [&] { return stop || (ln->busy && ln->job); });
      if (stop) return;
      b = std::move(ln->job);
      co = colls[b->coll];  // by value: collections may be added meanwhile
    }
    int32_t st = MV_OK;
    try {
      const size_t nx = (size_t)b->nq * co.d, nr = (size_t)b->nq * b->k;
      grow_pinned(reinterpret_cast<void**>(&ln->h_x), ln->cap_x, nx, sizeof(float));
      grow_pinned(reinterpret_cast<void**>(&ln->h_d), ln->cap_d, nr, sizeof(float));
      grow_pinned(reinterpret_cast<void**>(&ln->h_l), ln->cap_l, nr, sizeof(int64_t));
      size_t off = 0;
      for (Req* r : b->reqs) {
        std::memcpy(ln->h_x + off, r->x.data(), sizeof(float) * r->x.size());
        off += r->x.size();
      }
      ln->d_x.ensure(sizeof(float) * nx);
      ln->d_d.ensure(sizeof(float) * nr);
      ln->d_l.ensure(sizeof(int64_t) * nr);
      MV_CHECK_CUDA(cudaEventRecord(ln->ev_a, ln->s));
      MV_CHECK_CUDA(cudaMemcpyAsync(ln->d_x.p, ln->h_x, sizeof(float) * nx, cudaMemcpyHostToDevice, ln->s));
      if (co.kind == 0)
        st = mv_ivfpq_search_device(static_cast<mv_ivfpq*>(co.handle), ln->d_x.as<float>(), b->nq,
                                    b->k, nullptr, 0, &co.params, ln->d_d.as<float>(),
                                    ln->d_l.as<int64_t>(), ln->s);
      else if (co.kind == 1)
        st = mv_flat_search_device(static_cast<mv_flat*>(co.handle), ln->d_x.as<float>(), b->nq,
                                   b->k, nullptr, &co.params, ln->d_d.as<float>(),
                                   ln->d_l.as<int64_t>(), ln->s);
      else
        st = mv_sq8_search_device(static_cast<mv_sq8*>(co.handle), ln->d_x.as<float>(), b->nq, b->k,
                                  nullptr, co.rerank_factor, &co.params, ln->d_d.as<float>(),
                                  ln->d_l.as<int64_t>(), ln->s);
      if (st == MV_OK) {
        MV_CHECK_CUDA(cudaMemcpyAsync(ln->h_d, ln->d_d.p, sizeof(float) * nr, cudaMemcpyDeviceToHost, ln->s));
        MV_CHECK_CUDA(cudaMemcpyAsync(ln->h_l, ln->d_l.p, sizeof(int64_t) * nr, cudaMemcpyDeviceToHost, ln->s));
        MV_CHECK_CUDA(cudaEventRecord(ln->ev_b, ln->s));
        MV_CHECK_CUDA(cudaStreamSynchronize(ln->s));
        float t0 = 0.0f, t1 = 0.0f;
        if (cudaEventElapsedTime(&t0, ev_origin, ln->ev_a) == cudaSuccess &&
            cudaEventElapsedTime(&t1, ev_origin, ln->ev_b) == cudaSuccess) {
          std::lock_guard<std::mutex> lk(mu);
          if (intervals.size() >= 4096) intervals.erase(intervals.begin(), intervals.begin() + 2048);
          intervals.emplace_back(t0, t1);
        }
        size_t ro = 0;
        for (Req* r : b->reqs) {
          std::memcpy(r->out_d, ln->h_d + ro, sizeof(float) * r->nq * b->k);
          std::memcpy(r->out_l, ln->h_l + ro, sizeof(int64_t) * r->nq * b->k);
          ro += (size_t)r->nq * b->k;
        }
      }
    } catch (const mv::Error& e) {
      mv::set_last_error(e.what());
      st = e.code;
    } catch (const std::exception& e) {
      mv::set_last_error(e.what());
      st = MV_ERR_INTERNAL;
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      const auto now = clk::now();
      for (Req* r : b->reqs) finish(r, st, now);
      in_flight_bytes -= (int64_t)b->bytes;
      ln->busy = false;
    }
    cv_done.notify_all();
    cv_sched.notify_all();
  }
}

// Completes r (a whole request or a part of one); called with mu held.
void mv_server::finish(Req* r, int32_t st, clk::time_point now) {
  r->status = st;
  r->t_done = now;
  r->done = true;
  if (r->parent) {
    Req* p = r->parent;
    if (st != MV_OK && p->status == MV_OK) p->status = st;  // the first failure
    if (--p->parts_left > 0) return;
    p->t_done = now;
    p->done = true;
    // every part of p is finished: drop them (r among them; not used after)
    for (auto it = parts.begin(); it != parts.end();)
      it = (*it)->parent == p ? parts.erase(it) : it + 1;
  }
  ++completed;
}

extern "C" {

int32_t mv_server_create(mv_ctx* ctx, int64_t hbm_budget_bytes, int32_t lanes,
                         int64_t max_batch_queries, mv_server** out) {
  if (!ctx || !out || hbm_budget_bytes <= 0 || lanes <= 0 || lanes > 64 || max_batch_queries <= 0)
    return MV_ERR_ARG;
  *out = nullptr;
  try {
    cudaSetDevice(ctx->device);
    auto srv = std::make_unique<mv_server>();
    srv->ctx = ctx;
    srv->budget = hbm_budget_bytes;
    srv->max_batch = max_batch_queries;
    for (int i = 0; i < lanes; ++i) {
      auto ln = std::make_unique<Lane>();
      MV_CHECK_CUDA(cudaStreamCreateWithFlags(&ln->s, cudaStreamNonBlocking));
      MV_CHECK_CUDA(cudaEventCreate(&ln->ev_a));
      MV_CHECK_CUDA(cudaEventCreate(&ln->ev_b));
      srv->lanes.push_back(std::move(ln));
    }
    MV_CHECK_CUDA(cudaEventCreate(&srv->ev_origin));
    MV_CHECK_CUDA(cudaEventRecord(srv->ev_origin, srv->lanes[0]->s));
    MV_CHECK_CUDA(cudaEventSynchronize(srv->ev_origin));
    mv_server* p = srv.get();
    for (auto& ln : p->lanes) {
      Lane* l = ln.get();
      l->th = std::thread([p, l] { p->lane_loop(l); });
    }
    p->sched = std::thread([p] { p->sched_loop(); });
    *out = srv.release();
    return MV_OK;
  } catch (const mv::Error& e) {
    mv::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    mv::set_last_error(e.what());
    return MV_ERR_INTERNAL;
  }
}

int32_t mv_server_destroy(mv_server* srv) {
  if (!srv) return MV_ERR_ARG;
  {
    std::unique_lock<std::mutex> lk(srv->mu);
    // finish what is queued or in flight first
    srv->cv_done.wait(lk, [&] {
      if (!srv->queue.empty()) return false;
      for (auto& l : srv->lanes)
        if (l->busy) return false;
      return true;
    });
    srv->stop = true;
  }
  srv->cv_sched.notify_all();
  srv->cv_lane.notify_all();
  srv->sched.join();
  for (auto& l : srv->lanes) {
    l->th.join();
    if (l->h_x) cudaFreeHost(l->h_x);
    if (l->h_d) cudaFreeHost(l->h_d);
    if (l->h_l) cudaFreeHost(l->h_l);
    cudaEventDestroy(l->ev_a);
    cudaEventDestroy(l->ev_b);
    cudaStreamDestroy(l->s);
  }
  if (srv->ev_origin) cudaEventDestroy(srv->ev_origin);
  delete srv;
  return MV_OK;
}

static int32_t add_coll(mv_server* srv, Coll c, int32_t* id) {
  if (!srv || !c.handle || !id) return MV_ERR_ARG;
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->colls.push_back(c);
  *id = (int32_t)srv->colls.size() - 1;
  return MV_OK;
}

int32_t mv_server_add_ivfpq(mv_server* srv, mv_ivfpq* ix, const mv_search_params* params,
                            int32_t* id) {
  if (!ix) return MV_ERR_ARG;
  Coll c{};
  c.kind = 0;
  c.handle = ix;
  c.d = ix->d;
  if (params) c.params = *params;
  const int np = c.params.nprobe > 0 ? c.params.nprobe : ix->nprobe;
  // distance matrix or fused keys, probes, shortlist
  c.ws_per_query = (size_t)ix->nlist * 4 + (size_t)np * 8 + 4096 * 8 + 512;
  c.ws_fixed = 64ull << 20;
  return add_coll(srv, c, id);
}

int32_t mv_server_add_flat(mv_server* srv, mv_flat* ix, const mv_search_params* params,
                           int32_t* id) {
  if (!ix) return MV_ERR_ARG;
  Coll c{};
  c.kind = 1;
  c.handle = ix;
  c.d = ix->d;
  if (params) c.params = *params;
  c.ws_per_query = 64ull * 64 * 8 + 4096 * 8 + 1024;  // segment keys, shortlist
  c.ws_fixed = 1ull << 30;  // the plain form's distance tile
  return add_coll(srv, c, id);
}

int32_t mv_server_add_sq8(mv_server* srv, mv_sq8* ix, int32_t rerank_factor,
                          const mv_search_params* params, int32_t* id) {
  if (!ix || rerank_factor < 0) return MV_ERR_ARG;
  Coll c{};
  c.kind = 2;
  c.handle = ix;
  c.d = ix->d;
  if (params) c.params = *params;
  c.rerank_factor = rerank_factor;
  c.ws_per_query = 64ull * 64 * 8 + 4096 * 16 + (size_t)ix->dpad + 1024;
  c.ws_fixed = 1ull << 30;  // the integer scan's distance tile
  return add_coll(srv, c, id);
}

int32_t mv_server_submit(mv_server* srv, int32_t coll, const float* x, int64_t nq, int32_t k,
                         float* distances, int64_t* labels, int64_t* request_id) {
  if (!srv || !x || nq <= 0 || k <= 0 || k > 4096 || !distances || !labels || !request_id)
    return MV_ERR_ARG;
  std::unique_ptr<Req> r(new Req());
  std::vector<std::unique_ptr<Req>> parts;
  int d = 0;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    if (coll < 0 || coll >= (int32_t)srv->colls.size()) {
      mv::set_last_error("no such collection");
      return MV_ERR_ARG;
    }
    const Coll& c = srv->colls[coll];
    d = c.d;
    const int64_t part = std::min(nq, srv->max_batch);
    if ((int64_t)srv->estimate(c, part, k) > srv->budget) {
      mv::set_last_error("request larger than the server's memory budget");
      return MV_ERR_ARG;
    }
  }
  r->coll = coll;
  r->k = k;
  r->nq = nq;
  r->out_d = distances;
  r->out_l = labels;
  r->t_submit = clk::now();
  if (nq <= srv->max_batch) {
    r->x.assign(x, x + (size_t)nq * d);
  } else {
    // Parts of at most max_batch rows, each writing its own rows of the
    // caller's result arrays.
    for (int64_t q0 = 0; q0 < nq; q0 += srv->max_batch) {
      const int64_t n = std::min(srv->max_batch, nq - q0);
      std::unique_ptr<Req> pr(new Req());
      pr->coll = coll;
      pr->k = k;
      pr->nq = n;
      pr->x.assign(x + (size_t)q0 * d, x + (size_t)(q0 + n) * d);
      pr->out_d = distances + q0 * k;
      pr->out_l = labels + q0 * k;
      pr->t_submit = r->t_submit;
      pr->parent = r.get();
      parts.push_back(std::move(pr));
    }
    r->parts_left = (int)parts.size();
  }
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    r->id = srv->next_id++;
    *request_id = r->id;
    if (parts.empty()) {
      srv->queue.push_back(r.get());
    } else {
      for (auto& pr : parts) {
        pr->id = -r->id;
        srv->queue.push_back(pr.get());
        srv->parts.push_back(std::move(pr));
      }
    }
    srv->reqs.emplace(r->id, std::move(r));
  }
  srv->cv_sched.notify_all();
  return MV_OK;
}

// Waits for a request; returns its status and (optionally) its latency in
// seconds, then forgets it.
int32_t mv_server_wait(mv_server* srv, int64_t request_id, double* latency_s) {
  if (!srv) return MV_ERR_ARG;
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->reqs.find(request_id);
  if (it == srv->reqs.end()) return MV_ERR_ARG;
  Req* r = it->second.get();
  srv->cv_done.wait(lk, [&] { return r->done; });
  if (latency_s) latency_s[0] = std::chrono::duration<double>(r->t_done - r->t_submit).count();
  const int32_t st = r->status;
  srv->reqs.erase(it);
  return st;
}

// Peak number of batches whose device intervals (input copy to result copy)
// overlapped at one instant, over the recorded batches, and how many
// batches are recorded (the most recent few thousand).
int32_t mv_server_device_overlap(mv_server* srv, int64_t* out2) {
  if (!srv || !out2) return MV_ERR_ARG;
  std::vector<std::pair<float, int>> ev;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    for (const auto& iv : srv->intervals) {
      ev.emplace_back(iv.first, 1);
      ev.emplace_back(iv.second, -1);
    }
    out2[1] = (int64_t)srv->intervals.size();
  }
  // ends before starts at equal times: touching intervals do not overlap
  std::sort(ev.begin(), ev.end());
  int64_t cur = 0, peak = 0;
  for (const auto& e : ev) {
    cur += e.second;
    peak = std::max(peak, cur);
  }
  out2[0] = peak;
  return MV_OK;
}

int32_t mv_server_stats(mv_server* srv, int64_t* out4) {
  if (!srv || !out4) return MV_ERR_ARG;
  std::lock_guard<std::mutex> lk(srv->mu);
  out4[0] = srv->completed;
  out4[1] = srv->batches;
  out4[2] = srv->batched_queries;
  out4[3] = srv->peak_bytes;
  return MV_OK;
}

}  // extern "C"
